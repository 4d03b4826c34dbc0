// Allocation-free inner products: rtg_dots_noalloc.
//
// rtg_solve computes its Arnoldi inner products and residual norms from
// per-CTA partial sums, added in a fixed order, in a scratch buffer that the
// solver allocates on first use.  Some callers of
// this library may not allocate device memory at all: a host application
// whose memory manager owns every device allocation (a framework pool or a
// fixed budget set at start-up), or a driver that wraps its own Krylov loop
// around rtg_apply inside a region where cudaMalloc would stall or break the
// surrounding work (a latency-critical loop, a capture of a larger pipeline).
// For them this file provides the same kind of reduction (per-CTA partial
// sums, then a second launch that adds them in a fixed order) with its scratch
// in a file-scope device array: the caller passes inputs and outputs, and
// nothing is allocated.  Its grid and summation order are its own, so results
// can differ from the solver's in the last bits.
//
// Scratch: kNaBlocks x kNaMaxVectors doubles (296 x 64 x 8 B = 151,552 B) in
// g_noalloc_partial.  Every GPU that loads the library holds it until the
// process exits.  All calls share it: calls that overlap on the GPU (two
// streams, or two host threads) race on it and must be serialised by the
// caller.  Each call overwrites every partial sum it later reads, so no state
// from an earlier call survives into a result and nothing needs zeroing.
// The array's device address is cached per device for the life of the
// process: a cudaDeviceReset while the library is in use invalidates it (the
// module is reloaded at a new address), so the library must not be used
// across a reset.
#include <mutex>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kNaBlocks = 296;
constexpr int kNaThreads = 256;
constexpr int kNaMaxVectors = 64;
constexpr int kNaGroup = 8;
constexpr int kNaMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partial[kNaBlocks * kNaMaxVectors];

// Device address of g_noalloc_partial per device.  In host code the symbol
// name is only a host-side stand-in, so the address is looked up once per
// device with that device current.
double* g_partial_addr[kNaMaxDevices] = {nullptr};
std::mutex g_partial_mu;

double* partial_for_current_device() {
    int dev = 0;
    RTG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) throw RtgError{RTG_ERR_SIZE, "device index beyond 63"};
    std::lock_guard<std::mutex> lk(g_partial_mu);
    if (!g_partial_addr[dev]) {
        void* p = nullptr;
        RTG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partial));
        g_partial_addr[dev] = static_cast<double*>(p);
    }
    return g_partial_addr[dev];
}

// First stage: each CTA writes its partial sums of V_q . w for q < k.
__global__ void noalloc_dot_kernel(const double* __restrict__ V, int64_t ldv, int k,
                                   const double* __restrict__ w, int64_t n, double* __restrict__ partial) {
    __shared__ double red[kNaGroup][kNaThreads / 32];
    for (int g0 = 0; g0 < k; g0 += kNaGroup) {
        const int gk = min(kNaGroup, k - g0);
        double acc[kNaGroup];
#pragma unroll
        for (int q = 0; q < kNaGroup; ++q) acc[q] = 0.;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x) {
            const double wi = w[i];
#pragma unroll
            for (int q = 0; q < kNaGroup; ++q)
                if (q < gk) acc[q] += V[(int64_t)(g0 + q) * ldv + i] * wi;
        }
#pragma unroll
        for (int q = 0; q < kNaGroup; ++q) {
            double s = acc[q];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = s;
        }
        __syncthreads();
        if (threadIdx.x < gk) {
            double s = 0.;
            for (int wq = 0; wq < kNaThreads / 32; ++wq) s += red[threadIdx.x][wq];
            partial[(int64_t)blockIdx.x * k + g0 + threadIdx.x] = s;
        }
        __syncthreads();
    }
}

// Second stage: out[q] = sum over CTAs of the partial sums.
__global__ void noalloc_reduce_kernel(const double* __restrict__ partial, int nb, int k,
                                      double* __restrict__ out) {
    const int q = blockIdx.x;
    double s = 0.;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)b * k + q];
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.;
        for (int wq = 0; wq < (int)(blockDim.x + 31) / 32; ++wq) t += red[wq];
        out[q] = t;
    }
}

}  // namespace

}  // namespace rtg

using namespace rtg;

extern "C" int rtg_dots_noalloc(int k, const double* V, int64_t ldv, const double* w, int64_t n,
                                double* out, void* stream) {
    try {
        if (k < 1 || k > kNaMaxVectors)
            throw RtgError{RTG_ERR_SIZE, "k must be in [1, 64]: the static scratch holds 64 partial sums per CTA"};
        if (!V || !w || !out) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (n < 0) throw RtgError{RTG_ERR_ARG, "negative length"};
        if (k > 1 && ldv < n) throw RtgError{RTG_ERR_ARG, "ldv smaller than n"};
        double* partial = partial_for_current_device();
        cudaStream_t s = (cudaStream_t)stream;
        noalloc_dot_kernel<<<kNaBlocks, kNaThreads, 0, s>>>(V, ldv, k, w, n, partial), count_launch();
        noalloc_reduce_kernel<<<k, 256, 0, s>>>(partial, kNaBlocks, k, out), count_launch();
        RTG_CUDA(cudaGetLastError());
        return RTG_OK;
    } catch (const RtgError& e) {
        set_error(std::string("rtg_dots_noalloc: ") + e.msg);
        return e.code;
    }
}

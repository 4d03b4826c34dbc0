// Device-resident Krylov solvers for the split RT system A_II u_I = b
// (rt/solve.py:81-132).  Vectors stay full length (N) with the inflow-boundary
// entries held at zero, so every product is one masked operator apply.
//
//  * method 0 (plain): GMRES(m) in FP64, classical Gram-Schmidt Arnoldi (one
//    projection, PETSc's default), Givens on the device.
//  * method 1 (mixed): FP64 iterative refinement around FP32 GMRES(m): the
//    true residual r = b - A x is formed with the FP64 operator, the
//    correction A d = r is solved with FP32 applies and FP32 basis vectors
//    whose inner products accumulate in FP64; Hessenberg, Givens and the
//    convergence test are FP64.
//  * preconditioners 2 (sweep + column diffusion correction, rtg_coarse.cu)
//    and 3 (sweep + learned correction, rtg_nn.cu) run flexible GMRES: the
//    preconditioned vectors Z are kept and x += Z y, so the preconditioner is
//    applied once per iteration.  With preconditioner 3 a restart cycle that
//    cuts the residual by less than kStallRatio, or a refinement step whose
//    FP64 residual falls by less than kOuterStallRatio, switches the rest of
//    the solve to the sweep alone.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>
#include <tuple>
#include <type_traits>
#include <vector>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kRedBlocks = 1216;  // 8 per SM on 152 SMs: enough loads in flight for HBM; partial sums per reduction
constexpr int kRedThreads = 256;
constexpr int kDotGroup = 8;      // vectors per pass in multi_dot

// Arithmetic of the vector kernels: a vector's own precision per element and
// per warp (FP32 vectors stay on the FP32 pipe: GB300's FP64 rate is 1/64 of
// it), double from the per-warp sums on.
template <typename T>
using Acc = T;

// Sum over the blocks' partials of output q for one lane: the lane's blocks
// lane, lane + 32, ... loaded eight at a time (one L2 round trip per eight),
// added in that fixed order.
__device__ __forceinline__ double lane_partials(const double* __restrict__ partial, int nblocks, int stride, int q,
                                                int lane) {
    double sq = 0.;
    for (int b0 = lane; b0 < nblocks; b0 += 32 * 8) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int b = b0 + 32 * u;
            v[u] = b < nblocks ? __ldcg(partial + (int64_t)b * stride + q) : 0.;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) sq += v[u];
    }
    return sq;
}

// out[q] = <V_q, w> for q < k.  Each block writes its partial sums; the last
// block to finish (atomic ticket) adds them in block order, so the result does
// not depend on the schedule, writes out (and out_sum = out + add when add is
// given) and resets the ticket.
template <typename T>
__global__ void multi_dot_kernel(const T* __restrict__ V, int64_t ldv, int k, const T* __restrict__ w,
                                 int64_t n, double* __restrict__ partial, unsigned int* __restrict__ ticket,
                                 double* __restrict__ out, const double* __restrict__ add,
                                 double* __restrict__ out_sum, const int* __restrict__ stop) {
    __shared__ double red[kDotGroup][kRedThreads / 32];
    __shared__ int s_last;
    if (stop && *stop) return;   // every block: the ticket stays untouched
    for (int g0 = 0; g0 < k; g0 += kDotGroup) {
        const int gk = min(kDotGroup, k - g0);
        Acc<T> acc[kDotGroup];
#pragma unroll
        for (int q = 0; q < kDotGroup; ++q) acc[q] = Acc<T>(0);
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x) {
            const Acc<T> wi = w[i];
#pragma unroll
            for (int q = 0; q < kDotGroup; ++q)
                if (q < gk) acc[q] = fma(Acc<T>(V[(int64_t)(g0 + q) * ldv + i]), wi, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < kDotGroup; ++q) {
            Acc<T> sw = acc[q];
            for (int o = 16; o > 0; o >>= 1) sw += __shfl_down_sync(0xffffffffu, sw, o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = (double)sw;
        }
        __syncthreads();
        if (threadIdx.x < gk) {
            double sb = 0.;
            for (int wq = 0; wq < kRedThreads / 32; ++wq) sb += red[threadIdx.x][wq];
            partial[(int64_t)blockIdx.x * k + g0 + threadIdx.x] = sb;
        }
        __syncthreads();
    }
    __threadfence();   // every writer's partials before the ticket
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // one warp per output: lanes add every 32nd block, then a fixed shuffle tree
    const int lane = threadIdx.x & 31;
    for (int q = threadIdx.x >> 5; q < k; q += blockDim.x >> 5) {
        double sq = 0.;
        sq = lane_partials(partial, (int)gridDim.x, k, q, lane);
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
        if (lane == 0) {
            out[q] = sq;
            if (add) out_sum[q] = sq + add[q];
        }
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// Arnoldi step j (one thread): take the new Hessenberg column (projections
// hcol[0..j] and ||w||), apply the previous Givens rotations, form rotation j,
// update g and the residual estimate |g[j+1]|; slot[2j] = estimate,
// slot[2j+1] = stop code (0 go on, 1 converged or breakdown, 2 last allowed
// step, 3 non-finite); a nonzero code raises *stop so that the step after it
// does nothing.
struct ArnoldiState {
    const double* hcol;   // projections of the step
    double* H;
    double* cs;
    double* sn;
    double* g;
    double* slot;
    int* stop;
    const double* cyc;
    int j, ldh;
};

// hcol[0..j] are the projections, hjj1 = ||w|| the new subdiagonal entry
__device__ void arnoldi_update(const ArnoldiState a_st, const double* hcol, double hjj1) {
    const int j = a_st.j, ldh = a_st.ldh;
    double *H = a_st.H, *cs = a_st.cs, *sn = a_st.sn, *g = a_st.g, *slot = a_st.slot;
    int* stop = a_st.stop;
    const double tol = a_st.cyc[0];
    const bool last = j + 1 == (int)a_st.cyc[1];
    double* hc = H + (int64_t)j * ldh;
    for (int q = 0; q <= j; ++q) hc[q] = hcol[q];
    hc[j + 1] = hjj1;
    for (int q = 0; q < j; ++q) {
        const double a = hc[q], b = hc[q + 1];
        hc[q] = cs[q] * a + sn[q] * b;
        hc[q + 1] = -sn[q] * a + cs[q] * b;
    }
    const double a = hc[j], b = hc[j + 1];
    const double rr = hypot(a, b);
    cs[j] = rr > 0. ? a / rr : 1.;
    sn[j] = rr > 0. ? b / rr : 0.;
    hc[j] = rr;
    hc[j + 1] = 0.;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    const double est = fabs(g[j + 1]);
    int code = 0;
    if (!isfinite(est)) code = 3;
    else if (est <= tol || rr == 0.) code = 1;
    else if (last) code = 2;
    slot[2 * j] = est;
    slot[2 * j + 1] = (double)code;
    if (code) *stop = code;
}

// Fused Gram-Schmidt pass: w -= sum_{q<k} h[q] V_q, then out[0] = <w, w>
// and, for a device-driven step, the Arnoldi update, with one read of V and
// w.  Reductions as in multi_dot_kernel (last block, fixed order).
constexpr int kFuseMax = 32;   // vectors of the fused pass (longer bases use the separate kernels)

template <typename T>
__global__ void axpy_dot_kernel(T* __restrict__ w, const T* __restrict__ V, int64_t ldv, int k,
                                const double* __restrict__ h, int64_t n, double* __restrict__ partial,
                                unsigned int* __restrict__ ticket, double* __restrict__ out,
                                const int* __restrict__ stop, ArnoldiState ast) {
    constexpr int K = 1;
    if (stop && *stop) return;
    __shared__ Acc<T> hs[kFuseMax];
    __shared__ double red[K][kRedThreads / 32];
    __shared__ int s_last;
    if ((int)threadIdx.x < k) hs[threadIdx.x] = (Acc<T>)h[threadIdx.x];
    __syncthreads();
    const int nout = 1;
    Acc<T> acc[K];
#pragma unroll
    for (int q = 0; q < K; ++q) acc[q] = Acc<T>(0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        Acc<T> sv = w[i];
        // eight loads in flight before their FMAs (a plain loop waits for each)
        for (int q0 = 0; q0 < k; q0 += 8) {
            T vv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) vv[q] = q0 + q < k ? V[(int64_t)(q0 + q) * ldv + i] : T(0);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q0 + q < k) sv = fma(-hs[q0 + q], (Acc<T>)vv[q], sv);
        }
        w[i] = (T)sv;
        acc[0] = fma(sv, sv, acc[0]);
    }
#pragma unroll
    for (int q = 0; q < K; ++q) {
        if (q >= nout) break;
        Acc<T> sw = acc[q];
        for (int o = 16; o > 0; o >>= 1) sw += __shfl_down_sync(0xffffffffu, sw, o);
        if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = (double)sw;
    }
    __syncthreads();
    if ((int)threadIdx.x < nout) {
        double sb = 0.;
        for (int wq = 0; wq < kRedThreads / 32; ++wq) sb += red[threadIdx.x][wq];
        partial[(int64_t)blockIdx.x * nout + threadIdx.x] = sb;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int lane = threadIdx.x & 31;
    for (int q = threadIdx.x >> 5; q < nout; q += blockDim.x >> 5) {
        double sq = 0.;
        sq = lane_partials(partial, (int)gridDim.x, nout, q, lane);
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
        if (lane == 0) {
            out[q] = sq;
            // the norm pass of a device-driven step ends with the Arnoldi update
            if (ast.H) arnoldi_update(ast, ast.hcol, sqrt(sq));
        }
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// Sixteen bytes of T: the unit of the vectorised Gram-Schmidt kernels (one
// 128-bit load or store per basis vector and thread).
template <typename T>
struct alignas(16) Pack {
    static constexpr int n = 16 / (int)sizeof(T);
    T v[n];
};

template <typename T>
__device__ __forceinline__ Pack<T> load_pack(const T* p) {
    return *reinterpret_cast<const Pack<T>*>(p);
}

// Partial sums of one block (outputs q < nout, every thread's acc[q]) to
// partial[block * nout + q], then the last block to finish adds the blocks'
// partials in block order (the result does not depend on the schedule),
// writes out (and out_sum = out + add when add is given), runs the Arnoldi
// update after a norm pass that carries one, and resets the ticket.
template <typename T, int NO>
__device__ __forceinline__ void block_reduce_out(const T (&acc)[NO], int nout, double* __restrict__ partial,
                                                 unsigned int* __restrict__ ticket, double* __restrict__ out,
                                                 const double* __restrict__ add, double* __restrict__ out_sum,
                                                 const ArnoldiState* ast) {
    __shared__ double red[NO][kRedThreads / 32];
    __shared__ int s_last;
#pragma unroll
    for (int q = 0; q < NO; ++q) {
        if (q < nout) {
            T sw = acc[q];
            for (int o = 16; o > 0; o >>= 1) sw += __shfl_down_sync(0xffffffffu, sw, o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = (double)sw;
        }
    }
    __syncthreads();
    if ((int)threadIdx.x < nout) {
        double sb = 0.;
        for (int wq = 0; wq < kRedThreads / 32; ++wq) sb += red[threadIdx.x][wq];
        partial[(int64_t)blockIdx.x * nout + threadIdx.x] = sb;
    }
    __threadfence();   // every writer's partials before the ticket
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int lane = threadIdx.x & 31;
    for (int q = threadIdx.x >> 5; q < nout; q += blockDim.x >> 5) {
        double sq = lane_partials(partial, (int)gridDim.x, nout, q, lane);
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
        if (lane == 0) {
            out[q] = sq;
            if (add) out_sum[q] = sq + add[q];
            if (ast && ast->H) arnoldi_update(*ast, ast->hcol, sqrt(sq));
        }
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// Basis vectors whose packs a thread loads before their FMAs: all of them up
// to 16 (64 registers in either precision), eight at a time beyond that, so
// that two blocks of kRedThreads fit on an SM (128 registers a thread).
template <int KMAX>
__host__ __device__ constexpr int pack_group() { return KMAX <= 16 ? KMAX : 8; }

// multi_dot_kernel with 16-byte loads: out[q] = <V_q, w> for q < k <= KMAX.
// Each thread takes Pack<T>::n consecutive entries per step, the loads of up
// to 16 basis vectors issued before their FMAs; the last block also takes
// the entries past the last whole pack.  V_q and w start on 16-byte
// boundaries (the host checks).
template <typename T, int KMAX>
__global__ void __launch_bounds__(kRedThreads, 2) multi_dot_vec_kernel(
    const T* __restrict__ V, int64_t ldv, int k, const T* __restrict__ w, int64_t n, double* __restrict__ partial,
    unsigned int* __restrict__ ticket, double* __restrict__ out, const double* __restrict__ add,
    double* __restrict__ out_sum, const int* __restrict__ stop) {
    constexpr int P = Pack<T>::n;
    constexpr int G = pack_group<KMAX>();
    if (stop && *stop) return;   // every block: the ticket stays untouched
    T acc[KMAX];
#pragma unroll
    for (int q = 0; q < KMAX; ++q) acc[q] = T(0);
    const int64_t np = n / P;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < np; c += (int64_t)gridDim.x * blockDim.x) {
        const Pack<T> wp = load_pack(w + c * P);
#pragma unroll
        for (int q0 = 0; q0 < KMAX; q0 += G) {
            if (q0 >= k) break;
            Pack<T> vp[G];
#pragma unroll
            for (int u = 0; u < G; ++u)
                if (q0 + u < k) vp[u] = load_pack(V + (int64_t)(q0 + u) * ldv + c * P);
#pragma unroll
            for (int u = 0; u < G; ++u)
                if (q0 + u < k) {
#pragma unroll
                    for (int e = 0; e < P; ++e) acc[q0 + u] = fma(vp[u].v[e], wp.v[e], acc[q0 + u]);
                }
        }
    }
    if (blockIdx.x == gridDim.x - 1) {
        const int64_t i = np * P + threadIdx.x;
        if (i < n) {
            const T wi = w[i];
#pragma unroll
            for (int q = 0; q < KMAX; ++q)
                if (q < k) acc[q] = fma(V[(int64_t)q * ldv + i], wi, acc[q]);
        }
    }
    block_reduce_out<T, KMAX>(acc, k, partial, ticket, out, add, out_sum, nullptr);
}

// axpy_dot_kernel with 16-byte loads: w -= sum_{q<k} h[q] V_q, then
// out[0] = <w, w> and the Arnoldi update.  The update subtracts the terms in
// q order, as the scalar kernel does.
template <typename T, int KMAX>
__global__ void __launch_bounds__(kRedThreads, 2) axpy_dot_vec_kernel(
    T* __restrict__ w, const T* __restrict__ V, int64_t ldv, int k, const double* __restrict__ h, int64_t n,
    double* __restrict__ partial, unsigned int* __restrict__ ticket, double* __restrict__ out,
    const int* __restrict__ stop, ArnoldiState ast) {
    constexpr int P = Pack<T>::n;
    constexpr int NO = 1;
    constexpr int G = pack_group<KMAX>();
    if (stop && *stop) return;
    __shared__ T hs[KMAX];
    if ((int)threadIdx.x < k) hs[threadIdx.x] = (T)h[threadIdx.x];
    __syncthreads();
    T acc[NO];
#pragma unroll
    for (int q = 0; q < NO; ++q) acc[q] = T(0);
    const int64_t np = n / P;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < np; c += (int64_t)gridDim.x * blockDim.x) {
        Pack<T> sv = load_pack(w + c * P);
        Pack<T> vp[G];
#pragma unroll
        for (int q0 = 0; q0 < KMAX; q0 += G) {
            if (q0 >= k) break;
#pragma unroll
            for (int u = 0; u < G; ++u)
                if (q0 + u < k) vp[u] = load_pack(V + (int64_t)(q0 + u) * ldv + c * P);
#pragma unroll
            for (int u = 0; u < G; ++u)
                if (q0 + u < k) {
#pragma unroll
                    for (int e = 0; e < P; ++e) sv.v[e] = fma(-hs[q0 + u], vp[u].v[e], sv.v[e]);
                }
        }
        *reinterpret_cast<Pack<T>*>(w + c * P) = sv;
#pragma unroll
        for (int e = 0; e < P; ++e) acc[0] = fma(sv.v[e], sv.v[e], acc[0]);
    }
    if (blockIdx.x == gridDim.x - 1) {
        const int64_t i = np * P + threadIdx.x;
        if (i < n) {
            T si = w[i];
#pragma unroll
            for (int q = 0; q < KMAX; ++q)
                if (q < k) si = fma(-hs[q], V[(int64_t)q * ldv + i], si);
            w[i] = si;
            acc[0] = fma(si, si, acc[0]);
        }
    }
    block_reduce_out<T, NO>(acc, 1, partial, ticket, out, nullptr, nullptr, &ast);
}

// w -= sum_q h[q] V_q
template <typename T>
__global__ void multi_axpy_kernel(T* __restrict__ w, const T* __restrict__ V, int64_t ldv, int k,
                                  const double* __restrict__ h, int64_t n) {
    __shared__ Acc<T> hs[64];
    if (threadIdx.x < k) hs[threadIdx.x] = (Acc<T>)h[threadIdx.x];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        Acc<T> sv = w[i];
        for (int q0 = 0; q0 < k; q0 += 8) {
            T vv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) vv[q] = q0 + q < k ? V[(int64_t)(q0 + q) * ldv + i] : T(0);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q0 + q < k) sv = fma(-hs[q0 + q], Acc<T>(vv[q]), sv);
        }
        w[i] = (T)sv;
    }
}

// out = w / sqrt(nrm2sq[0]); hcol[k] = sqrt(nrm2sq[0]).  zfill (optional): the
// next sweep's output, filled with the sentinel, and its claim counter reset,
// so that the sweep needs no fill launch of its own.
template <typename T>
__global__ void normalize_kernel(const T* __restrict__ w, T* __restrict__ out, const double* nrm2sq,
                                 double* hcol, int k, int64_t n, const int* __restrict__ stop,
                                 T* __restrict__ zfill = nullptr, unsigned int* __restrict__ next = nullptr) {
    using U = typename Sentinel<T>::U;
    if (stop && *stop) return;
    // one FP64 square root and division per block (GB300's FP64 rate is low)
    __shared__ Acc<T> s_inv;
    if (threadIdx.x == 0) {
        const double nr = sqrt(nrm2sq[0]);
        if (blockIdx.x == 0) {
            hcol[k] = nr;
            if (zfill) *next = 0u;
        }
        s_inv = (Acc<T>)(nr > 0. ? 1. / nr : 0.);
    }
    __syncthreads();
    const Acc<T> inv = s_inv;
    U* zq = reinterpret_cast<U*>(zfill);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        out[i] = (T)(Acc<T>(w[i]) * inv);
        if (zq) zq[i] = Sentinel<T>::bits;
    }
}

// Start of a restart cycle on the device: g = (beta, 0, ...) with beta = ||r||
// from *beta_dev, cyc = (tolerance, steps allowed this cycle, beta, code) for
// the Arnoldi update and the host; a residual already within tolerance (code 1)
// or non-finite (code 3) raises *stop at once, otherwise it is cleared.
__global__ void cycle_init_kernel(double* __restrict__ g, int n, const double* __restrict__ beta_dev,
                                  int* __restrict__ stop, double* __restrict__ cyc, double tol, int steps) {
    const double beta = *beta_dev;
    for (int q = threadIdx.x; q < n; q += blockDim.x) g[q] = q == 0 ? beta : 0.;
    if (threadIdx.x == 0) {
        const int code = !isfinite(beta) ? 3 : (beta <= tol ? 1 : 0);
        *stop = code;
        cyc[0] = tol;
        cyc[1] = (double)steps;
        cyc[2] = beta;
        cyc[3] = (double)code;
    }
}

// y = H^{-1} g for the j x j upper-triangular Hessenberg factor (one thread)
__global__ void ysolve_kernel(const double* __restrict__ H, int ldh, const double* __restrict__ g, int j,
                              double* __restrict__ y) {
    for (int q = j - 1; q >= 0; --q) {
        double sacc = g[q];
        for (int c = q + 1; c < j; ++c) sacc -= H[(int64_t)c * ldh + q] * y[c];
        y[q] = sacc / H[(int64_t)q * ldh + q];
    }
}

// y = a*x + b*y over full vectors of possibly different types (FP32 when both
// are FP32, else FP64); a zero coefficient drops its term without reading it
// (the buffer may hold anything, NaN included)
template <typename TX, typename TY>
__global__ void axpby_kernel(double a, const TX* __restrict__ x, double b, TY* __restrict__ y, int64_t n) {
    using A = typename std::conditional<sizeof(TX) == 4 && sizeof(TY) == 4, float, double>::type;
    const A aa = (A)a, bb = (A)b;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (TY)((a == 0. ? A(0) : aa * (A)x[i]) + (b == 0. ? A(0) : bb * (A)y[i]));
}

// x += scale * sum_q c[q] V_q (c on device; FP32 when both vectors are FP32)
template <typename TV, typename TX>
__global__ void combine_kernel(TX* __restrict__ x, const TV* __restrict__ V, int64_t ldv, int k,
                               const double* __restrict__ c, double scale, int64_t n) {
    using A = typename std::conditional<sizeof(TV) == 4 && sizeof(TX) == 4, float, double>::type;
    __shared__ A cs[64];
    if (threadIdx.x < k) cs[threadIdx.x] = (A)c[threadIdx.x];
    __syncthreads();
    const A sc = (A)scale;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        A sv = A(0);
        for (int q = 0; q < k; ++q) sv = fma(cs[q], (A)V[(int64_t)q * ldv + i], sv);
        x[i] = (TX)((A)x[i] + sc * sv);
    }
}

constexpr double kStallRatio = 0.9;
constexpr double kOuterStallRatio = 0.5;

inline int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)std::min<int64_t>(g, 152 * 8);
}

}  // namespace

struct Workspace {
    int m = 0;
    int64_t N = 0;
    int64_t ld = 0;          // stride of the bases: N rounded up to 64 entries (16-byte aligned vectors)
    double* V64 = nullptr;   // (m+1) x ld
    float* V32 = nullptr;    // (m+1) x ld
    double *b = nullptr, *r = nullptr, *x = nullptr, *t = nullptr, *gb = nullptr;
    double *w64 = nullptr, *z64 = nullptr, *t64 = nullptr;
    float *w32 = nullptr, *d32 = nullptr, *z32 = nullptr, *t32 = nullptr, *s32 = nullptr;
    double* Z64 = nullptr;      // m x ld flexible basis (every preconditioned mode)
    float* Z32 = nullptr;
    // grids of the 16-byte Gram-Schmidt kernels (blocks resident on every SM,
    // at most kRedBlocks): [FP64][KMAX 8, 16, 32] and [FP64][KMAX][norm pass]
    int gdot[2][3] = {};
    int gaxd[2][3] = {};
    double* partial = nullptr;  // kRedBlocks x (m+1)
    unsigned int* ticket = nullptr;   // last-block ticket of multi_dot_kernel (0 between launches)
    // device Arnoldi state of the lagged-check inner loop
    int* stop = nullptr;
    double *dH = nullptr, *dcs = nullptr, *dsn = nullptr, *dg = nullptr, *dslot = nullptr;
    double* hslot = nullptr;          // pinned: per step estimate and code
    std::vector<cudaEvent_t> ev;      // one per step
    double* cyc = nullptr;            // device: tolerance and steps of the current cycle
    // graphs of one inner step, by (value size, preconditioner mode, step, restart length)
    std::map<std::tuple<int, int, int, int>, std::pair<cudaGraphExec_t, long long>> graphs;   // exec, kernels
    cudaStream_t cap = nullptr;       // capture stream
    bool warm[2] = {false, false};    // a cycle ran uncaptured (plans and launch shapes exist), per precision
    double* hdev = nullptr;     // y of the cycle's update [m+2], (unused) [m+2], projections [m+2], nrm [1]
    double* hhost = nullptr;    // pinned
    // the last Arnoldi cycle with at least one step: its j x j triangular
    // factor R (Givens-reduced Hessenberg, columns m + 1 apart) is in dH
    // (device loop) or in hlast (host loop)
    int last_j = 0;
    bool last_on_device = false;
    // per column: 1 when its rows of A mask_B g are zero for every g (neither
    // it nor a face neighbour holds an inflow-boundary node)
    int32_t* rhs_skip = nullptr;
    std::vector<double> hlast;
    std::vector<void*> allocs;
};

namespace {

template <typename T>
T* dalloc(Workspace* ws, int64_t n) {
    void* p = nullptr;
    RTG_CUDA(cudaMalloc(&p, sizeof(T) * (size_t)std::max<int64_t>(n, 1)));
    ws->allocs.push_back(p);
    return (T*)p;
}

void init_vec_grids(Workspace* ws);

Workspace* get_ws(rtg_handle* h, int m) {
    Workspace* ws = h->ws;
    const int64_t N = h->host.ndof;
    if (ws && ws->m >= m && ws->N == N) return ws;
    free_workspace(h);
    ws = new Workspace();
    h->ws = ws;
    ws->m = m;
    ws->N = N;
    ws->ld = (N + 63) / 64 * 64;
    ws->V64 = dalloc<double>(ws, (int64_t)(m + 1) * ws->ld);
    ws->V32 = dalloc<float>(ws, (int64_t)(m + 1) * ws->ld);
    init_vec_grids(ws);
    ws->b = dalloc<double>(ws, N);
    ws->r = dalloc<double>(ws, N);
    ws->x = dalloc<double>(ws, N);
    ws->t = dalloc<double>(ws, N);
    ws->gb = dalloc<double>(ws, N);
    ws->w64 = dalloc<double>(ws, N);
    ws->w32 = dalloc<float>(ws, N);
    ws->d32 = dalloc<float>(ws, N);
    ws->z64 = dalloc<double>(ws, N);
    ws->t64 = dalloc<double>(ws, N);
    ws->z32 = dalloc<float>(ws, N);
    ws->t32 = dalloc<float>(ws, N);
    ws->s32 = dalloc<float>(ws, N);
    ws->partial = dalloc<double>(ws, (int64_t)kRedBlocks * (m + 2));
    ws->ticket = dalloc<unsigned int>(ws, 1);
    RTG_CUDA(cudaMemset(ws->ticket, 0, sizeof(unsigned int)));
    ws->stop = dalloc<int>(ws, 1);
    RTG_CUDA(cudaMemset(ws->stop, 0, sizeof(int)));
    ws->dH = dalloc<double>(ws, (int64_t)(m + 1) * m);
    ws->dcs = dalloc<double>(ws, m);
    ws->dsn = dalloc<double>(ws, m);
    ws->dg = dalloc<double>(ws, m + 1);
    ws->dslot = dalloc<double>(ws, 2 * m);
    ws->cyc = dalloc<double>(ws, 4);
    RTG_CUDA(cudaMallocHost(&ws->hslot, sizeof(double) * (2 * m + 2)));   // steps, then beta and start code
    ws->ev.assign(m, nullptr);
    for (auto& e : ws->ev) RTG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ws->hdev = dalloc<double>(ws, 4 * (m + 2));
    RTG_CUDA(cudaMallocHost(&ws->hhost, sizeof(double) * 4 * (m + 2)));
    return ws;
}

// blocks of kernel fn resident on all SMs of the current device, at most kRedBlocks
int resident_grid(const void* fn) {
    int dev = 0, sms = 0, per_sm = 0;
    RTG_CUDA(cudaGetDevice(&dev));
    RTG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kRedThreads, 0));
    return std::max(1, std::min(kRedBlocks, per_sm * sms));
}

// the grids of every 16-byte Gram-Schmidt kernel, found once per workspace
// (outside any stream capture)
void init_vec_grids(Workspace* ws) {
    ws->gdot[0][0] = resident_grid((const void*)multi_dot_vec_kernel<float, 8>);
    ws->gdot[0][1] = resident_grid((const void*)multi_dot_vec_kernel<float, 16>);
    ws->gdot[0][2] = resident_grid((const void*)multi_dot_vec_kernel<float, 32>);
    ws->gdot[1][0] = resident_grid((const void*)multi_dot_vec_kernel<double, 8>);
    ws->gdot[1][1] = resident_grid((const void*)multi_dot_vec_kernel<double, 16>);
    ws->gdot[1][2] = resident_grid((const void*)multi_dot_vec_kernel<double, 32>);
    ws->gaxd[0][0] = resident_grid((const void*)axpy_dot_vec_kernel<float, 8>);
    ws->gaxd[0][1] = resident_grid((const void*)axpy_dot_vec_kernel<float, 16>);
    ws->gaxd[0][2] = resident_grid((const void*)axpy_dot_vec_kernel<float, 32>);
    ws->gaxd[1][0] = resident_grid((const void*)axpy_dot_vec_kernel<double, 8>);
    ws->gaxd[1][1] = resident_grid((const void*)axpy_dot_vec_kernel<double, 16>);
    ws->gaxd[1][2] = resident_grid((const void*)axpy_dot_vec_kernel<double, 32>);
}

// the 16-byte kernels take vectors that start on 16-byte boundaries, ldv apart
template <typename T>
bool packed(const T* p, int64_t ldv) {
    return ((uintptr_t)p & 15u) == 0 && (ldv * (int64_t)sizeof(T)) % 16 == 0;
}

inline int kmax_index(int k) { return k <= 8 ? 0 : (k <= 16 ? 1 : 2); }   // KMAX 8, 16, 32

// out[q] = <V_q, w> for q < k (and out_sum = out + add when add is given)
template <typename T>
void dots(Workspace* ws, const T* V, int64_t ldv, int k, const T* w, int64_t n, double* out,
          const double* add, double* out_sum, cudaStream_t s, const int* stop = nullptr) {
    if (k > 32 || !packed(V, ldv) || !packed(w, 0)) {
        multi_dot_kernel<T><<<kRedBlocks, kRedThreads, 0, s>>>(V, ldv, k, w, n, ws->partial, ws->ticket, out, add,
                                                              out_sum, stop), count_launch();
        return;
    }
    const int ki = kmax_index(k);
    const int g = ws->gdot[sizeof(T) == 8][ki];
    if (ki == 0)
        multi_dot_vec_kernel<T, 8><<<g, kRedThreads, 0, s>>>(V, ldv, k, w, n, ws->partial, ws->ticket, out, add,
                                                             out_sum, stop);
    else if (ki == 1)
        multi_dot_vec_kernel<T, 16><<<g, kRedThreads, 0, s>>>(V, ldv, k, w, n, ws->partial, ws->ticket, out, add,
                                                              out_sum, stop);
    else
        multi_dot_vec_kernel<T, 32><<<g, kRedThreads, 0, s>>>(V, ldv, k, w, n, ws->partial, ws->ticket, out, add,
                                                              out_sum, stop);
    count_launch();
}

// w -= V h over k <= 32 vectors fused with out[0] = <w, w> and the Arnoldi
// update of ast
template <typename T>
void axpy_dot(Workspace* ws, T* w, const T* V, int64_t ldv, int k, const double* h, int64_t n, double* out,
              const int* stop, ArnoldiState ast, cudaStream_t s) {
    if (!packed(V, ldv) || !packed((const T*)w, 0)) {
        axpy_dot_kernel<T><<<kRedBlocks, kRedThreads, 0, s>>>(w, V, ldv, k, h, n, ws->partial, ws->ticket, out, stop,
                                                             ast), count_launch();
        return;
    }
    const int ki = kmax_index(k);
    const int g = ws->gaxd[sizeof(T) == 8][ki];
    if (ki == 0)
        axpy_dot_vec_kernel<T, 8><<<g, kRedThreads, 0, s>>>(w, V, ldv, k, h, n, ws->partial, ws->ticket, out, stop,
                                                            ast);
    else if (ki == 1)
        axpy_dot_vec_kernel<T, 16><<<g, kRedThreads, 0, s>>>(w, V, ldv, k, h, n, ws->partial, ws->ticket, out, stop,
                                                             ast);
    else
        axpy_dot_vec_kernel<T, 32><<<g, kRedThreads, 0, s>>>(w, V, ldv, k, h, n, ws->partial, ws->ticket, out, stop,
                                                             ast);
    count_launch();
}

template <typename T>
const OpView<T>& view(const rtg_handle* h);
template <>
const OpView<double>& view<double>(const rtg_handle* h) { return h->v64; }
template <>
const OpView<float>& view<float>(const rtg_handle* h) { return h->v32; }

double norm2(rtg_handle* h, Workspace* ws, const double* v, cudaStream_t s) {
    dots<double>(ws, v, 0, 1, v, ws->N, ws->hdev, nullptr, nullptr, s);
    RTG_CUDA(cudaMemcpyAsync(ws->hhost, ws->hdev, sizeof(double), cudaMemcpyDeviceToHost, s));
    RTG_CUDA(cudaStreamSynchronize(s));
    return std::sqrt(ws->hhost[0]);
}

// r = b - A_II x (FP64), returns ||r||
double residual64(rtg_handle* h, Workspace* ws, const double* b, const double* x, double* r,
                  cudaStream_t s) {
    launch_apply<double>(h, h->v64, RTG_SYSTEM | RTG_MASK_ROWS, x, r, s);
    axpby_kernel<double, double><<<grid_for(ws->N), 256, 0, s>>>(1., b, -1., r, ws->N), count_launch();
    return norm2(h, ws, r, s);
}

struct GmresResult {
    int iters = 0;
    bool converged = false;
    double res = 0.;
};

struct PcState {
    int mode = 0;        // 0 none, 1 sweep, 2 sweep + diffusion, 3 sweep + learned (2, 3 flexible)
    int sweeps = 0;
    int coarse = 0;
    int learned = 0;
    int fallbacks = 0;
};

template <typename T>
T* flex_basis(Workspace* ws, int m);
template <>
double* flex_basis<double>(Workspace* ws, int m) {
    if (!ws->Z64) ws->Z64 = dalloc<double>(ws, (int64_t)m * ws->ld);
    return ws->Z64;
}
template <>
float* flex_basis<float>(Workspace* ws, int m) {
    if (!ws->Z32) ws->Z32 = dalloc<float>(ws, (int64_t)m * ws->ld);
    return ws->Z32;
}

// GMRES(m) for A_II d = r0 in precision T starting from d = 0.  rhs is given
// in T (scaled); stops when the estimated residual <= tol_abs or after
// max_it iterations.  Returns the solution in xT (T).  hist gets estimates.
//
// Inner loop: the Givens rotations and the convergence test run on the
// device (at the end of the norm pass), and the host reads step j's outcome only after it
// has queued step j+1, so the GPU never waits for the host between steps.
// A step that follows the last one finds *stop raised and every launch of it
// returns at once.  The two-level preconditioner (mode 2) and restart lengths
// above the fused Gram-Schmidt limit keep a host check per step.
template <typename T>
GmresResult gmres(rtg_handle* h, Workspace* ws, const T* rhs, T* xT, T* wbuf, T* V, int m,
                  double tol_abs, int max_it, std::vector<double>* hist, int* applies,
                  PcState& pc, cudaStream_t s) {
    const int64_t N = ws->N;
    const int64_t ld = ws->ld;
    GmresResult res;
    const OpView<T>& v = view<T>(h);
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    axpby_kernel<T, T><<<grid_for(N), 256, 0, s>>>(0., rhs, 0., xT, N), count_launch();
    // r = rhs - A x = rhs (x = 0)
    int total = 0;
    bool first = true;
    double* ho = ws->hdev + 2 * (m + 2);
    double* nr = ws->hdev + 3 * (m + 2);
    while (total < max_it) {
        // r = rhs - A x  into V_0 (unnormalised), beta = ||r||
        if (first) {
            axpby_kernel<T, T><<<grid_for(N), 256, 0, s>>>(1., rhs, 0., wbuf, N), count_launch();
        } else {
            launch_apply<T>(h, v, RTG_SYSTEM | RTG_MASK_ROWS, xT, wbuf, s);
            ++*applies;
            axpby_kernel<T, T><<<grid_for(N), 256, 0, s>>>(1., rhs, -1., wbuf, N), count_launch();
        }
        first = false;
        dots<T>(ws, wbuf, 0, 1, wbuf, N, nr, nullptr, nullptr, s);
        const int mode = pc.mode;   // fixed for the cycle
        // every preconditioned mode keeps M(v_j) (for the sweep alone this is
        // right preconditioning: x += Z y = P^{-1} V y without a last sweep)
        const bool flex = mode >= 1;
        T* Z = flex ? flex_basis<T>(ws, ws->m) : nullptr;
        // the normalisation that makes v_j also prepares the sweep of z_j
        unsigned int* next = flex ? sweep_counter(h, s) : nullptr;
        normalize_kernel<T><<<grid_for(N), 256, 0, s>>>(wbuf, V, nr, ho, 0, N, nullptr, Z, next), count_launch();
        const bool lagged = mode != 2 && m <= kFuseMax;
        double beta = 0.;
        if (!lagged) {
            RTG_CUDA(cudaMemcpyAsync(ws->hhost, ho, sizeof(double), cudaMemcpyDeviceToHost, s));
            RTG_CUDA(cudaStreamSynchronize(s));
            beta = ws->hhost[0];
            res.res = beta;
            if (!std::isfinite(beta)) throw RtgError{RTG_ERR_NONFINITE, "non-finite residual in GMRES"};
            if (beta <= tol_abs) {
                res.converged = true;
                break;
            }
        }
        const int* stop = lagged ? ws->stop : nullptr;
        OpView<T> vs = v;
        vs.stop = stop;
        // counts of one step
        auto count_step = [&](int times) {
            if (flex) pc.sweeps += times;
            if (mode == 2) pc.coarse += times;
            if (mode == 3) pc.learned += times;
            *applies += times * (mode == 2 ? 2 : 1);
        };
        // one Arnoldi step on stream s: w = A M(v_j), CGS2 against V, v_{j+1} = w / ||w||
        // (with a device Arnoldi state the norm pass ends with the Arnoldi update)
        auto step = [&](int j, cudaStream_t s, ArnoldiState ast) {
            T* vj = V + (int64_t)j * ld;
            T* vn = V + (int64_t)(j + 1) * ld;
            if (flex) {
                T* zj = Z + (int64_t)j * ld;
                apply_sweep<T>(h, vj, zj, s, nullptr, nullptr, stop, true);
                if (mode == 2) {
                    apply_coarse<T>(h, vj, zj, s);
                } else if (mode == 3) {
                    apply_learned<T>(h, zj, s, stop);
                }
                launch_apply<T>(h, vs, RTG_SYSTEM | RTG_MASK_ROWS, zj, wbuf, s);
            } else {
                launch_apply<T>(h, vs, RTG_SYSTEM | RTG_MASK_ROWS, vj, wbuf, s);
            }
            // classical Gram-Schmidt, one projection, as PETSc's GMRES does by
            // default (KSPGMRESClassicalGramSchmidtOrthogonalization without
            // refinement; the reference's rt/solve.py:80-100 calls it): ho =
            // V^T w, then w -= V ho with ||w||^2.  On the two-scatterer problem
            // it takes the iterations and reaches the errors of two projections
            // in both precisions (one read of V per step less)
            dots<T>(ws, V, ld, j + 1, wbuf, N, ho, nullptr, nullptr, s, stop);
            if (j + 1 <= kFuseMax) {
                axpy_dot<T>(ws, wbuf, V, ld, j + 1, ho, N, nr, stop, ast, s);
            } else {
                multi_axpy_kernel<T><<<grid_for(N), 256, 0, s>>>(wbuf, V, ld, j + 1, ho, N), count_launch();
                dots<T>(ws, wbuf, 0, 1, wbuf, N, nr, nullptr, nullptr, s);
            }
            T* zn = (flex && j + 1 < m) ? Z + (int64_t)(j + 1) * ld : nullptr;
            normalize_kernel<T><<<grid_for(N), 256, 0, s>>>(wbuf, vn, nr, ho, j + 1, N, stop, zn, zn ? next : nullptr),
                count_launch();
        };
        int j = 0;   // steps of this cycle that count
        if (lagged) {
            const int steps = std::min(m, max_it - total);
            cycle_init_kernel<<<1, 64, 0, s>>>(ws->dg, m + 1, ho, ws->stop, ws->cyc, tol_abs, steps),
                count_launch();
            RTG_CUDA(cudaMemcpyAsync(ws->hslot + 2 * m, ws->cyc + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
            double* start = ws->hslot + 2 * m;   // beta, start code (read with step 0's outcome)
            const int pi = sizeof(T) == 8 ? 1 : 0;
            auto full_step = [&](int q, cudaStream_t st) {
                ArnoldiState ast{ho, ws->dH, ws->dcs, ws->dsn, ws->dg, ws->dslot, ws->stop, ws->cyc, q, m + 1};
                step(q, st, ast);
            };
            int issued = 0, code = 0;
            for (int q = 0; q < steps; ++q) {
                if (ws->warm[pi]) {
                    // replay the captured step (captured on first use)
                    const auto key = std::make_tuple((int)sizeof(T), mode, q, m);
                    auto it = ws->graphs.find(key);
                    if (it == ws->graphs.end()) {
                        if (!ws->cap) RTG_CUDA(cudaStreamCreateWithFlags(&ws->cap, cudaStreamNonBlocking));
                        cudaGraph_t graph;
                        const long long n0 = launch_counter().load();
                        RTG_CUDA(cudaStreamBeginCapture(ws->cap, cudaStreamCaptureModeThreadLocal));
                        try {
                            full_step(q, ws->cap);
                        } catch (...) {
                            cudaGraph_t broken = nullptr;
                            cudaStreamEndCapture(ws->cap, &broken);
                            if (broken) cudaGraphDestroy(broken);
                            throw;
                        }
                        RTG_CUDA(cudaStreamEndCapture(ws->cap, &graph));
                        // recorded launches are counted when the graph runs
                        const long long nk = launch_counter().load() - n0;
                        launch_counter().fetch_sub(nk);
                        cudaGraphExec_t exec;
                        RTG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
                        RTG_CUDA(cudaGraphDestroy(graph));
                        it = ws->graphs.emplace(key, std::make_pair(exec, nk)).first;
                    }
                    RTG_CUDA(cudaGraphLaunch(it->second.first, s));
                    launch_counter().fetch_add(it->second.second);
                } else {
                    full_step(q, s);
                }
                count_step(1);
                RTG_CUDA(cudaMemcpyAsync(ws->hslot + 2 * q, ws->dslot + 2 * q, 2 * sizeof(double),
                                         cudaMemcpyDeviceToHost, s));
                RTG_CUDA(cudaEventRecord(ws->ev[q], s));
                issued = q + 1;
                if (q >= 1) {
                    RTG_CUDA(cudaEventSynchronize(ws->ev[q - 1]));   // start[] is valid from here on
                    if (start[1] > 0.) break;                        // the cycle had nothing to do
                    code = (int)ws->hslot[2 * (q - 1) + 1];
                    if (code > 0) {
                        j = q;   // steps 0 .. q-1 count; step q ran as a no-op
                        break;
                    }
                }
            }
            if (code <= 0) {
                RTG_CUDA(cudaEventSynchronize(ws->ev[issued - 1]));
                if (!(start[1] > 0.)) {
                    code = (int)ws->hslot[2 * (issued - 1) + 1];
                    j = issued;
                }
            }
            beta = start[0];
            if (start[1] > 0.) {
                // the residual was already within tolerance (or not finite): no step counts
                count_step(-issued);
                res.res = beta;
                if ((int)start[1] == 3) throw RtgError{RTG_ERR_NONFINITE, "non-finite residual in GMRES"};
                res.converged = true;
                break;
            }
            // undo the counts of a step that did nothing
            count_step(-(issued - j));
            ws->warm[pi] = true;
            if (code == 3) throw RtgError{RTG_ERR_NONFINITE, "non-finite residual in GMRES"};
            for (int q = 0; q < j; ++q)
                if (hist) hist->push_back(ws->hslot[2 * q]);
            total += j;
            res.res = ws->hslot[2 * (j - 1)];
            res.converged = res.res <= tol_abs;
            ws->last_j = j;
            ws->last_on_device = true;
            // y = H^{-1} g on the device (into hdev, where the combine reads it)
            ysolve_kernel<<<1, 1, 0, s>>>(ws->dH, m + 1, ws->dg, j, ws->hdev), count_launch();
        } else {
            std::fill(g.begin(), g.end(), 0.);
            g[0] = beta;
            for (; j < m && total < max_it; ++j) {
                step(j, s, ArnoldiState{});
                count_step(1);
                RTG_CUDA(cudaMemcpyAsync(ws->hhost, ws->hdev, sizeof(double) * 3 * (m + 2),
                                         cudaMemcpyDeviceToHost, s));
                RTG_CUDA(cudaStreamSynchronize(s));
                ++total;
                double* hc = &H[(size_t)j * (m + 1)];
                for (int q = 0; q <= j; ++q) hc[q] = ws->hhost[2 * (m + 2) + q];
                hc[j + 1] = ws->hhost[2 * (m + 2) + j + 1];
                // Givens
                for (int q = 0; q < j; ++q) {
                    const double a = hc[q], b = hc[q + 1];
                    hc[q] = cs[q] * a + sn[q] * b;
                    hc[q + 1] = -sn[q] * a + cs[q] * b;
                }
                const double a = hc[j], b = hc[j + 1];
                const double rr = std::hypot(a, b);
                cs[j] = rr > 0. ? a / rr : 1.;
                sn[j] = rr > 0. ? b / rr : 0.;
                hc[j] = rr;
                hc[j + 1] = 0.;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
                const double est = std::fabs(g[j + 1]);
                if (!std::isfinite(est)) throw RtgError{RTG_ERR_NONFINITE, "non-finite residual in GMRES"};
                if (hist) hist->push_back(est);
                res.res = est;
                if (est <= tol_abs || rr == 0.) {
                    ++j;
                    res.converged = est <= tol_abs;
                    break;
                }
            }
        }
        if (!lagged && j > 0) {
            ws->last_j = j;
            ws->last_on_device = false;
            ws->hlast.assign(H.begin(), H.begin() + (size_t)j * (m + 1));
        }
        if (!lagged) {
            // y = H^{-1} g (upper triangular j x j)
            for (int q = j - 1; q >= 0; --q) {
                double sacc = g[q];
                for (int c = q + 1; c < j; ++c) sacc -= H[(size_t)c * (m + 1) + q] * y[c];
                y[q] = sacc / H[(size_t)q * (m + 1) + q];
            }
            RTG_CUDA(cudaMemcpyAsync(ws->hdev, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        }
        if (flex) {
            // x += Z y
            combine_kernel<T, T><<<grid_for(N), 256, 0, s>>>(xT, Z, ld, j, ws->hdev, 1., N), count_launch();
        } else {
            combine_kernel<T, T><<<grid_for(N), 256, 0, s>>>(xT, V, ld, j, ws->hdev, 1., N), count_launch();
        }
        res.iters = total;
        if (res.converged) break;
        if (mode == 3 && !(res.res < kStallRatio * beta)) {
            pc.mode = 1;   // the learned correction stalled this cycle
            ++pc.fallbacks;
        }
    }
    res.iters = total;
    return res;
}

// Precond 3 trial: from the same right-hand side, one cycle of kTrialSteps
// steps with the sweep alone and one with the learned correction; the
// correction stays when its log residual reduction per second is larger.  The
// pair runs twice and only the second round is timed, so that first-use costs
// (apply autotuning, sweep tables, graph captures) fall in the first.  Runs
// once per handle and inner precision (h->nn_trial), the first time precond 3
// meets a residual; adds its work to pc and applies.
constexpr int kTrialSteps = 8;

template <typename T>
void learned_trial(rtg_handle* h, Workspace* ws, const T* rhs, double beta, T* xT, T* wbuf, T* V, int* applies,
                   PcState& pc, int* trial_its, cudaStream_t s) {
    const int pi = sizeof(T) == 8 ? 0 : 1;
    cudaEvent_t e0, e1;
    RTG_CUDA(cudaEventCreate(&e0));
    RTG_CUDA(cudaEventCreate(&e1));
    double rate[2] = {0., 0.};   // log reduction per second: sweep alone, with the correction
    try {
        for (int qq = 0; qq < 4; ++qq) {
            const int q = qq & 1;
            PcState t;
            t.mode = q == 0 ? 1 : 3;
            RTG_CUDA(cudaEventRecord(e0, s));
            GmresResult gr = gmres<T>(h, ws, rhs, xT, wbuf, V, kTrialSteps, 0., kTrialSteps, nullptr, applies, t, s);
            RTG_CUDA(cudaEventRecord(e1, s));
            RTG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            RTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            const double ratio = std::max(gr.res / beta, 1e-30);
            rate[q] = -std::log(ratio) / std::max(1e-3 * (double)ms, 1e-9);
            pc.sweeps += t.sweeps;
            pc.learned += t.learned;
            *trial_its += gr.iters;
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->nn_trial[pi] = rate[1] > rate[0] ? 1 : 2;
}

}  // namespace

int last_hessenberg(rtg_handle* h, double* R, int cap, int* n, cudaStream_t s) {
    Workspace* ws = h->ws;
    const int j = ws ? ws->last_j : 0;
    *n = j;
    if (!R || j == 0) return RTG_OK;
    if (cap < j * j) throw RtgError{RTG_ERR_SIZE, "R needs n*n doubles"};
    const int ld = ws->m + 1;
    std::vector<double> raw((size_t)j * ld);
    if (ws->last_on_device) {
        RTG_CUDA(cudaMemcpyAsync(raw.data(), ws->dH, sizeof(double) * raw.size(), cudaMemcpyDeviceToHost, s));
        RTG_CUDA(cudaStreamSynchronize(s));
    } else {
        std::copy(ws->hlast.begin(), ws->hlast.begin() + raw.size(), raw.begin());
    }
    // column-major j x j, the rows below the diagonal zero
    for (int c = 0; c < j; ++c)
        for (int q = 0; q < j; ++q) R[(size_t)c * j + q] = q <= c ? raw[(size_t)c * ld + q] : 0.;
    return RTG_OK;
}

void free_workspace(rtg_handle* h) {
    if (!h->ws) return;
    for (void* p : h->ws->allocs) cudaFree(p);
    if (h->ws->hhost) cudaFreeHost(h->ws->hhost);
    if (h->ws->hslot) cudaFreeHost(h->ws->hslot);
    for (cudaEvent_t e : h->ws->ev)
        if (e) cudaEventDestroy(e);
    for (auto& kv : h->ws->graphs) cudaGraphExecDestroy(kv.second.first);
    if (h->ws->cap) cudaStreamDestroy(h->ws->cap);
    delete h->ws;
    h->ws = nullptr;
}

int solve(rtg_handle* h, const double* f, const double* g, double* u, const rtg_solve_opts* o,
          rtg_solve_info* info, double* hist, int hist_cap, cudaStream_t s) {
    const auto t0 = std::chrono::steady_clock::now();
    const int m = std::max(1, std::min(o->restart, 60));
    Workspace* ws = get_ws(h, m);
    const int64_t N = ws->N;
    rtg_solve_info inf{};
    std::vector<double> hv;

    // b = mask_I (f - A mask_B g)     (rt/solve.py:98-101).  mask_B g is zero
    // outside the inflow-boundary nodes, so only their columns and the
    // columns facing them get nonzero rows: the apply runs on those alone
    // (the same kernels, the same bits) into a zeroed t.
    if (!ws->rhs_skip) {
        const HostTables& t = h->host;
        const int nc = (int)t.cols.size();
        std::vector<char> inflow(nc, 0);
        for (const ElemDev& E : t.elems)
            if (E.flags >> 4) inflow[E.col] = 1;
        std::vector<int32_t> skip(nc, 1);
        for (int c = 0; c < nc; ++c) {
            bool need = inflow[c];
            for (int q = 0; q < 8 && !need; ++q) {
                const int nb = t.col_nbr8[(size_t)8 * c + q];
                need = nb >= 0 && inflow[nb];
            }
            skip[c] = need ? 0 : 1;
        }
        ws->rhs_skip = dalloc<int32_t>(ws, nc);
        RTG_CUDA(cudaMemcpy(ws->rhs_skip, skip.data(), sizeof(int32_t) * nc, cudaMemcpyHostToDevice));
    }
    launch_mask_vector(h, 1, g, ws->gb, s);
    RTG_CUDA(cudaMemsetAsync(ws->t, 0, sizeof(double) * N, s));
    {
        OpView<double> vb = h->v64;
        vb.skip = ws->rhs_skip;
        launch_apply<double>(h, vb, RTG_SYSTEM | RTG_MASK_ROWS, ws->gb, ws->t, s);
    }
    inf.fp64_applies++;
    launch_mask_vector(h, 0, f, ws->b, s);
    axpby_kernel<double, double><<<grid_for(N), 256, 0, s>>>(-1., ws->t, 1., ws->b, N), count_launch();
    // x0 = u_I (nonzero guess) or 0; the reference starts from f_I (rt/solve.py:104)
    if (o->nonzero_guess)
        launch_mask_vector(h, 0, u, ws->x, s);
    else
        axpby_kernel<double, double><<<grid_for(N), 256, 0, s>>>(0., ws->b, 0., ws->x, N), count_launch();

    inf.rhs_norm = norm2(h, ws, ws->b, s);
    const double tol = std::max(o->rtol * inf.rhs_norm, o->atol);
    double res;
    if (o->nonzero_guess) {
        res = residual64(h, ws, ws->b, ws->x, ws->r, s);
        inf.fp64_applies++;
    } else {
        // x0 = 0: r0 = b, no apply
        axpby_kernel<double, double><<<grid_for(N), 256, 0, s>>>(1., ws->b, 0., ws->r, N), count_launch();
        res = inf.rhs_norm;
    }
    inf.res0 = res;
    hv.push_back(res);
    int applies32 = 0, applies64 = 0;
    PcState pc;
    pc.mode = o->precond;
    if (pc.mode < 0 || pc.mode > 3) throw RtgError{RTG_ERR_ARG, "unknown preconditioner"};
    if (pc.mode == 3 && !nn_has_params(h))
        throw RtgError{RTG_ERR_ARG, "preconditioner 3 needs a network (rtg_nn_set_params)"};
    if (pc.mode >= 1) get_sweep(h, s);
    if (pc.mode == 2 && !h->coarse) build_coarse(h, s);
    const int tpi = o->method == 0 ? 0 : 1;
    // precond 3 after a lost trial: the sweep alone
    auto trial_verdict = [&]() {
        if (pc.mode == 3 && h->nn_trial[tpi] == 2) {
            pc.mode = 1;
            ++pc.fallbacks;
        }
    };
    trial_verdict();

    if (o->method == 0) {
        // GMRES on the correction: A d = r, x += d, repeated until converged.
        int used = 0;
        while (res > tol && used < o->max_it) {
            if (pc.mode == 3 && h->nn_trial[0] == 0) {
                learned_trial<double>(h, ws, ws->r, res, ws->w64, ws->t, ws->V64, &applies64, pc, &inf.trial_its, s);
                trial_verdict();
            }
            GmresResult gr = gmres<double>(h, ws, ws->r, ws->w64, ws->t, ws->V64, m, tol,
                                           o->max_it - used, &hv, &applies64, pc, s);
            used += std::max(gr.iters, 1);
            axpby_kernel<double, double><<<grid_for(N), 256, 0, s>>>(1., ws->w64, 1., ws->x, N), count_launch();
            const double prev = res;
            res = residual64(h, ws, ws->b, ws->x, ws->r, s);
            inf.fp64_applies++;
            hv.push_back(res);
            if (gr.iters == 0) break;
            if (pc.mode == 3 && !(res < kOuterStallRatio * prev)) {
                pc.mode = 1;
                ++pc.fallbacks;
            }
        }
        inf.iterations = used;
    } else {
        int used = 0, outer = 0;
        const int max_outer = o->max_outer > 0 ? o->max_outer : 20;
        const double inner_rtol = o->inner_rtol > 0. ? o->inner_rtol : 1e-6;
        while (res > tol && used < o->max_it && outer < max_outer) {
            // r32 = r / ||r||
            axpby_kernel<double, float><<<grid_for(N), 256, 0, s>>>(1. / res, ws->r, 0., ws->w32, N), count_launch();
            if (pc.mode == 3 && h->nn_trial[1] == 0) {
                learned_trial<float>(h, ws, ws->w32, 1., ws->d32, ws->s32, ws->V32, &applies32, pc, &inf.trial_its, s);
                trial_verdict();
            }
            // one FP32 solve per refinement step, capped at 20 restart cycles
            const int inner_cap = std::min(o->max_it - used, 20 * m);
            GmresResult gr = gmres<float>(h, ws, ws->w32, ws->d32, ws->s32, ws->V32, m,
                                          std::max(inner_rtol, tol / res), inner_cap,
                                          nullptr, &applies32, pc, s);
            used += std::max(gr.iters, 1);
            axpby_kernel<float, double><<<grid_for(N), 256, 0, s>>>(res, ws->d32, 1., ws->x, N), count_launch();
            const double prev = res;
            res = residual64(h, ws, ws->b, ws->x, ws->r, s);
            inf.fp64_applies++;
            hv.push_back(res);
            ++outer;
            if (pc.mode == 3 && !(res < kOuterStallRatio * prev)) {
                pc.mode = 1;   // the FP64 residual stalled: the sweep alone from here on
                ++pc.fallbacks;
            }
        }
        inf.iterations = used;
        inf.outer = outer;
    }
    inf.fp64_applies += applies64;
    inf.fp32_applies += applies32;
    inf.sweeps = pc.sweeps;
    inf.learned = pc.learned;
    inf.coarse = pc.coarse;
    inf.fallbacks = pc.fallbacks;
    inf.learned_kept = (o->precond == 3 && h->nn_trial[tpi] == 1) ? 1 : 0;
    if (o->precond >= 1 && sweep_status(h, s) != RTG_OK)
        throw RtgError{RTG_ERR_TIMEOUT, "a sweep wait gave up; the solution is not valid"};
    if (apply_status(h, s) != RTG_OK)
        throw RtgError{RTG_ERR_TIMEOUT, "a tensor-core wait gave up; the solution is not valid and the handle "
                                        "must be destroyed"};
    inf.res_f = res;
    inf.converged = res <= tol ? 1 : 0;
    // u = x on the unknowns, g on the inflow-boundary DOFs (rt/solve.py:163)
    axpby_kernel<double, double><<<grid_for(N), 256, 0, s>>>(1., ws->x, 1., ws->gb, N), count_launch();
    RTG_CUDA(cudaMemcpyAsync(u, ws->gb, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    RTG_CUDA(cudaStreamSynchronize(s));
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    inf.hist_len = (int)std::min<size_t>(hv.size(), hist ? (size_t)hist_cap : 0);
    if (hist)
        for (int q = 0; q < inf.hist_len; ++q) hist[q] = hv[q];
    if (info) *info = inf;
    return RTG_OK;
}

}  // namespace rtg

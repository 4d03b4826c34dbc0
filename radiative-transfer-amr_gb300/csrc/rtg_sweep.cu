// Upwind block transport sweep used as the preconditioner of the RT solve.
//
// P is the block-lower-triangular part of the transport operator (streaming
// plus total extinction, no scattering) in an upwind element order:
//   * element-diagonal block, per angular node r of the element: the
//     (nx ny) x (nx ny) matrix of extinction, minus interior streaming, plus
//     the outflow face terms (the same entries rtg_apply uses with
//     RTG_SYSTEM).  All scattering, including the same-direction term, is
//     left to the Krylov iteration: with a forward-peaked phase function on a
//     coarse angular cell the same-direction term can exceed the extinction
//     and make the block singular;
//   * off-diagonal blocks: the inflow face couplings to neighbour elements
//     that come earlier in the order.
// Elements are ordered by Kahn levels of the "depends on the upwind
// neighbour" graph over all angular cells at once; where the graph has a
// cycle (cells that lie in no single quadrant couple on every face) the
// couplings that close it are dropped from P.  One persistent launch applies
// P^{-1}: CTAs take elements in level order and wait on the upwind values
// themselves (z is filled with a sentinel first).  An element whose upwind
// map G_e = -B_e C_e (built once, FP64 with an FP32 copy) fits in shared
// memory computes z_e = B_e rin_e + G_e z_upwind in one phase after its
// inputs arrive; the others form the face couplings in factorised form
// (T = Et z, c = Es T) and apply the face columns of B_e.
// Applying P^{-1} is exact for the transport part of an acyclic mesh; the
// cross-cell scattering is left to the Krylov iteration.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <queue>
#include <unordered_map>
#include <vector>

#include <cuda_bf16.h>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kSweepThreads = 256;
constexpr size_t kSweepSmemBudget = 110 * 1024;  // rhs + prefetched block inverse (2 CTAs per SM)
constexpr size_t kSweepSmemSmall = 72 * 1024;    // the alternatives the first sweep also times (3 CTAs per SM)
constexpr size_t kSweepSmemTiny = 54 * 1024;     // ... and 4 CTAs per SM (the register limit): more copies in flight
constexpr int kSweepShapes = 5;
// the shapes the first sweep times: (threads per CTA, shared-memory budget);
// the 128-thread CTAs fit 6 or 8 per SM, each staging one element
constexpr int kShapeThreads[kSweepShapes] = {kSweepThreads, kSweepThreads, kSweepThreads, 128, 128};
constexpr size_t kShapeBudget[kSweepShapes] = {kSweepSmemBudget, kSweepSmemSmall, kSweepSmemTiny, 36 * 1024,
                                               27 * 1024};
constexpr int kMaxCplStaged = 32;               // active couplings staged per element
constexpr int kMaxBlock = 100;  // nx*ny supported by the element-block inverse

__device__ __forceinline__ int gofs_s(int n) { return (n - 1) * n * (2 * n - 1) / 6; }

__device__ __forceinline__ bool bdry_node_s(int bm, int i, int j, int nx, int ny) {
    return ((bm & 1) && i == nx - 1) || ((bm & 2) && j == ny - 1) || ((bm & 4) && i == 0) ||
           ((bm & 8) && j == 0);
}

// One CTA per (element, angular node): assemble the element block for that
// node in shared memory as [A | I] and invert it by Gauss-Jordan elimination
// with partial pivoting.  Rows of inflow-boundary nodes become identity rows.
// The elimination runs in FP32 (GB300's FP64 rate would make large meshes take
// minutes); the inverse only defines the preconditioner, a fixed linear
// operator, so the FP64 solve still converges to FP64 accuracy.
__global__ void build_block_inverse_kernel(OpView<float> v, const int32_t* __restrict__ blk_elem,
                                           const int32_t* __restrict__ blk_r,
                                           const int64_t* __restrict__ blk_off, double* __restrict__ inv64,
                                           float* __restrict__ inv32, int* __restrict__ status) {
    extern __shared__ float smemf[];
    const int b = blockIdx.x;
    const int e = blk_elem[b];
    const int r = blk_r[b];
    const ElemDev E = v.elems[e];
    const ColDev C = v.cols[E.col];
    const int nx = C.nx, ny = C.ny, nn = nx * ny, nth = E.nth;
    const int ld = 2 * nn;
    float* M = smemf;                      // nn x 2nn
    __shared__ int piv;
    __shared__ float pval;
    const float* A = v.ang + E.ang;
    const float* Gx = v.G + gofs_s(nx);
    const float* Gy = v.G + gofs_s(ny);
    const float* wxs = v.lglw + nx * kMaxNodes;
    const float* wys = v.lglw + ny * kMaxNodes;
    const float mc = v.econst[4 * e], icx = v.econst[4 * e + 1], icy = v.econst[4 * e + 2];
    const float wsr = A[nth + r], wcr = A[2 * nth + r], wr = A[r];
    const int bm = E.flags >> 4;
    for (int k = threadIdx.x; k < nn * ld; k += blockDim.x) {
        const int row = k / ld, col = k % ld;
        const int p = row / ny, q = row % ny;
        const bool bd = ((bm & 1) && p == nx - 1) || ((bm & 2) && q == ny - 1) || ((bm & 4) && p == 0) ||
                        ((bm & 8) && q == 0);
        float val = 0.f;
        if (col >= nn) {
            val = (col - nn == row) ? 1.f : 0.f;
        } else if (bd) {
            val = (col == row) ? 1.f : 0.f;
        } else {
            const int i = col / ny, j = col % ny;
            const int node = C.node_off + col;
            if (col == row) {
                val += mc * wr * v.kw[node];
                for (int F = 0; F < 4; ++F) {
                    if (!(E.flags & (1 << F))) continue;
                    const bool on = (F == 0 && p == nx - 1) || (F == 1 && q == ny - 1) || (F == 2 && p == 0) ||
                                    (F == 3 && q == 0);
                    if (!on) continue;
                    const float dc = (F % 2 == 0) ? icy : icx;
                    const float w = (F % 2 == 0) ? wys[q] : wxs[p];
                    val += dc * w * wr * A[(3 + F) * nth + r];
                }
            }
            if (p == i) val -= icx * wxs[p] * wsr * Gy[q * ny + j];
            if (q == j) val -= icy * wys[q] * wcr * Gx[p * nx + i];
        }
        M[k] = val;
    }
    __syncthreads();
    for (int k = 0; k < nn; ++k) {
        if (threadIdx.x < 32) {
            // partial pivoting: warp-wide arg-max of |M[i][k]| over i >= k
            // (ties go to the lowest row, as a serial scan would)
            float bv = -1.f;
            int best = k;
            for (int i = k + threadIdx.x; i < nn; i += 32) {
                const float a = fabsf(M[i * ld + k]);
                if (a > bv) {
                    bv = a;
                    best = i;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const float ov = __shfl_down_sync(0xffffffffu, bv, o);
                const int oi = __shfl_down_sync(0xffffffffu, best, o);
                if (ov > bv || (ov == bv && oi < best)) {
                    bv = ov;
                    best = oi;
                }
            }
            if (threadIdx.x == 0) {
                piv = best;
                pval = M[best * ld + k];
                if (!(bv > 0.f)) atomicExch(status, 1);
            }
        }
        __syncthreads();
        if (piv != k)
            for (int c = threadIdx.x; c < ld; c += blockDim.x) {
                const float t = M[k * ld + c];
                M[k * ld + c] = M[piv * ld + c];
                M[piv * ld + c] = t;
            }
        __syncthreads();
        const float inv = pval != 0.f ? 1.f / pval : 0.f;
        for (int c = threadIdx.x; c < ld; c += blockDim.x) M[k * ld + c] *= inv;
        __syncthreads();
        for (int t = threadIdx.x; t < nn * ld; t += blockDim.x) {
            const int i = t / ld, c = t % ld;
            if (i == k || c == k) continue;
            M[t] -= M[i * ld + k] * M[k * ld + c];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nn; i += blockDim.x)
            if (i != k) M[i * ld + k] = 0.f;
        __syncthreads();
    }
    // stored transposed, [input node k][output node ij], so that the sweep's
    // threads (consecutive ij, same angular node) read consecutive entries
    double* o64 = inv64 + blk_off[b];
    float* o32 = inv32 + blk_off[b];
    for (int t = threadIdx.x; t < nn * nn; t += blockDim.x) {
        const int k = t / nn, ij = t % nn;
        const float val = M[ij * ld + nn + k];
        o64[t] = (double)val;
        o32[t] = val;
    }
}

// Persistent wavefront sweep: z_e = B_e^{-1} (rin_e - sum_upwind C_ee' z_e').
// CTAs claim elements in topological order from an atomic counter.  Before
// the sweep z is filled with a sentinel (a NaN payload that arithmetic never
// produces); an element reads the upwind face lines it needs straight from z,
// spinning (bounded) on each value until it no longer holds the sentinel.  A
// value that has arrived is both the data and the signal, so there is no flag,
// no release fence and no second round trip per level.  The upwind elements
// come earlier in the claim order, so they were claimed by CTAs that are
// already running and every wait ends unless a CTA gave up; a CTA that gives
// up sets *status and every other CTA stops waiting as soon as it sees it.
//
// The critical path of the sweep is the work an element does after its wait,
// so everything that does not depend on upwind values happens before it: the
// block inverse, the residual, the mortar matrices and, by linearity,
//     zpre = B rin                         (before the wait)
//     z    = zpre - B c,  c = couplings    (after the wait)
// where c is nonzero only on the face nodes that have active couplings, so the
// second product runs over those face columns of B only.  The couplings are
// factorised per neighbour: T[jj][r] = sum_a Et[a][r] zl[jj][a], then
// c[q][r] = sum_neighbours dcoeff sum_jj Es[jj][q] T[jj][r].
constexpr long long kSpinLimitCycles = 2000000000LL;  // about one second
constexpr int kMaxFaceNodes = 4 * kMaxNodes;
constexpr int kTr = 8;   // trace entries per element

// Element records.  Everything an element reads about itself before its data
// (its scalars, the active couplings with their staging offsets, the face
// nodes those couplings reach, the one-phase map fields) is resolved at set-up
// and stored per claim index with a fixed stride, so that the claim is
// followed by one coalesced load instead of a chain of dependent ones.
// int32 words; 64-bit values take two words, low first.
constexpr int kRecE = 0;        // element
constexpr int kRecCol = 1;      // column
constexpr int kRecDof = 2;      // first DOF (two words)
constexpr int kRecNx = 4, kRecNy = 5, kRecNth = 6;
constexpr int kRecFlags = 7;    // ElemDev::flags
constexpr int kRecInv = 8;      // first block-inverse entry (two words)
constexpr int kRecNcs = 10;     // staged active couplings; -1: read from global memory
constexpr int kRecNf = 11;      // face nodes with active couplings
constexpr int kRecCplB = 12, kRecCplE = 13;   // the element's couplings (all of them)
constexpr int kRecOk = 14;      // one-phase path: bit 0 FP32, bit 1 FP64
constexpr int kRecReg = 15;     // one-phase staged region in values, FP32 then FP64
constexpr int kRecNup = 17;     // upwind values of the one-phase map
constexpr int kRecGoff = 18;    // map offset, FP32 (two words) then FP64 (two words)
constexpr int kRecUoff = 22;    // upwind index list offset (two words)
constexpr int kRecDirect = 24;  // 1: every staged coupling has diagonal mortars (Es and Et)
constexpr int kRecHead = 25;
// per staged coupling: face, m1, nth1, n0, stride, es, et, base (two words),
// staging offset, coupling index, (unused); then the face nodes (ascending ij)
constexpr int kRecCpl = 12;
constexpr int kCplF = 0, kCplM1 = 1, kCplNt1 = 2, kCplN0 = 3, kCplStr = 4, kCplEs = 5, kCplEt = 6, kCplBase = 7,
              kCplOff = 9, kCplK = 10,
              kCplDiag = 11;   // bit 0: Es diagonal, bit 1: Et diagonal (off-diagonal entries below 1e-13 of the largest)
constexpr int kRecMax = kRecHead + kRecCpl * kMaxCplStaged + kMaxFaceNodes;

__device__ __forceinline__ int64_t rec64(const int* w) {
    return (int64_t)(((uint64_t)(uint32_t)w[1] << 32) | (uint64_t)(uint32_t)w[0]);
}

// hash of a key of 64-bit words (the bits of an element's block inputs)
struct WordsHash {
    size_t operator()(const std::vector<uint64_t>& v) const {
        uint64_t h = 1469598103934665603ull;
        for (uint64_t w : v) {
            h ^= w + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
            h *= 1099511628211ull;
        }
        return (size_t)h;
    }
};


__device__ __forceinline__ float from_bits_f(unsigned int u) { return __uint_as_float(u); }
__device__ __forceinline__ double from_bits_f(unsigned long long u) { return __longlong_as_double((long long)u); }

template <typename T>
__device__ __forceinline__ T from_bits(typename Sentinel<T>::U u) {
    return from_bits_f(u);
}

// Relaxed GPU-scope accesses: morally strong, so a reader racing with the
// writer sees either the sentinel or the whole published value.
__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int* p) {
    unsigned int u;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(u) : "l"(p) : "memory");
    return u;
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long u;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(u) : "l"(p) : "memory");
    return u;
}
__device__ __forceinline__ void st_relaxed(float* p, float x) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(x)) : "memory");
}
__device__ __forceinline__ void st_relaxed(double* p, double x) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"((unsigned long long)__double_as_longlong(x))
                 : "memory");
}

// Load a value of z that an upwind element publishes during this sweep:
// spin (bounded) while it still holds the sentinel.  Returns false when the
// wait gave up (timeout, or another CTA's status).  The poll is one L2 round
// trip per iteration: the status word and the clock are checked every 16th
// iteration only, so they do not add a second round trip to each poll.
template <typename T>
__device__ __forceinline__ bool load_published(const T* p, T& out, int* status) {
    using U = typename Sentinel<T>::U;
    const U* q = reinterpret_cast<const U*>(p);
    U u = ld_relaxed(q);
    if (u != Sentinel<T>::bits) {
        out = from_bits<T>(u);
        return true;
    }
    const long long t0 = clock64();
    for (unsigned it = 1;; ++it) {
        u = ld_relaxed(q);
        if (u != Sentinel<T>::bits) {
            out = from_bits<T>(u);
            return true;
        }
        if ((it & 15u) == 0u) {
            if (__ldcv(status) != 0) return false;
            if (clock64() - t0 > kSpinLimitCycles) {
                atomicExch(status, RTG_ERR_TIMEOUT);
                return false;
            }
        }
    }
}

// Starts a sweep: resets the claim counter and writes the sentinel over the
// values of z the sweep will publish (elements of columns left out keep their
// values).  Device-side, so that a captured graph can replay it.
template <typename T>
__global__ void sweep_fill_kernel(OpView<T> v, int ne, T* __restrict__ z, unsigned int* __restrict__ next) {
    using U = typename Sentinel<T>::U;
    if (v.stop && *v.stop) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) *next = 0u;
    U* q = reinterpret_cast<U*>(z);
    for (int e = blockIdx.x; e < ne; e += gridDim.x) {
        const ElemDev E = v.elems[e];
        if (v.skip && v.skip[E.col]) continue;
        const ColDev C = v.cols[E.col];
        const int nloc = C.nx * C.ny * E.nth;
        for (int t = threadIdx.x; t < nloc; t += blockDim.x) q[E.dof_off + t] = Sentinel<T>::bits;
    }
}

// Storage of the upwind maps a sweep reads: BF16 for the FP32 sweep (like the
// block inverses: the map only defines the preconditioner, a fixed linear
// operator), FP64 for the FP64 sweep.  Entries are widened to T on use.
template <typename T>
struct MapStore;
template <>
struct MapStore<float> {
    using type = __nv_bfloat16;
};
template <>
struct MapStore<double> {
    using type = double;
};

// Row length (entries) of an element's upwind map in the sweep of precision
// T: nup rounded up so that a row is a whole number of 16-byte units of the
// stored type and the number of units is odd (rows of consecutive outputs
// then start in different 16-byte bank groups, so 16-byte loads of a quarter
// warp do not conflict).
template <typename T>
__host__ __device__ __forceinline__ int map_ld(int nup) {
    constexpr int kVec = 16 / (int)sizeof(typename MapStore<T>::type);
    if (nup <= 0) return 0;
    int r = (nup + kVec - 1) / kVec * kVec;
    if ((r / kVec) % 2 == 0) r += kVec;
    return r;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool on_face(int F, int i, int j, int nx, int ny) {
    return (F == 0 && i == nx - 1) || (F == 1 && j == ny - 1) || (F == 2 && i == 0) || (F == 3 && j == 0);
}

// Upwind maps of the elements that take the one-phase path: for element e
// with nup upwind values (the facing node lines of its active couplings, in
// coupling order, then jj, then a), G_e = -B_e C_e maps them to the element's
// values: z_e = B_e rin_e + G_e z_upwind.  G is stored by output row
// (l = ij*nth + r), each row map_ld<T>(nup) values long (zero padded), each
// element's block on a 16-byte boundary; FP32 and FP64 copies have their own
// offsets.  Shared memory of the path (after rhs and zpre): upwind values
// [map_ld, zero padded] | G_e [nloc * map_ld] | B_e [nth*nn*nn].
// acc + sum over 16-byte units q0 <= q < q1 of a map row times the upwind
// values (16-byte loads; four independent partial sums in FP32, two in FP64)
__device__ __forceinline__ float map_row(const float* g, const float* zl, int q0, int q1, float acc) {
    float a0 = acc, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    const float4* g4 = reinterpret_cast<const float4*>(g);
    const float4* z4 = reinterpret_cast<const float4*>(zl);
    for (int q = q0; q < q1; ++q) {
        const float4 gv = g4[q], zv = z4[q];
        a0 = fmaf(gv.x, zv.x, a0);
        a1 = fmaf(gv.y, zv.y, a1);
        a2 = fmaf(gv.z, zv.z, a2);
        a3 = fmaf(gv.w, zv.w, a3);
    }
    return (a0 + a1) + (a2 + a3);
}
// BF16 map (the FP32 sweep): a 16-byte unit holds eight entries, widened to
// FP32 against two 16-byte units of upwind values
__device__ __forceinline__ float map_row(const __nv_bfloat16* g, const float* zl, int q0, int q1, float acc) {
    float a0 = acc, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    const uint4* g4 = reinterpret_cast<const uint4*>(g);
    const float4* z4 = reinterpret_cast<const float4*>(zl);
    for (int q = q0; q < q1; ++q) {
        const uint4 gv = g4[q];
        const float4 za = z4[2 * q], zb = z4[2 * q + 1];
        const float2 g01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&gv.x));
        const float2 g23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&gv.y));
        const float2 g45 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&gv.z));
        const float2 g67 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&gv.w));
        a0 = fmaf(g01.x, za.x, a0);
        a1 = fmaf(g01.y, za.y, a1);
        a2 = fmaf(g23.x, za.z, a2);
        a3 = fmaf(g23.y, za.w, a3);
        a0 = fmaf(g45.x, zb.x, a0);
        a1 = fmaf(g45.y, zb.y, a1);
        a2 = fmaf(g67.x, zb.z, a2);
        a3 = fmaf(g67.y, zb.w, a3);
    }
    return (a0 + a1) + (a2 + a3);
}
__device__ __forceinline__ double map_row(const double* g, const double* zl, int q0, int q1, double acc) {
    double a0 = acc, a1 = 0.;
    const double2* g2 = reinterpret_cast<const double2*>(g);
    const double2* z2 = reinterpret_cast<const double2*>(zl);
    for (int q = q0; q < q1; ++q) {
        const double2 gv = g2[q], zv = z2[q];
        a0 = fma(gv.x, zv.x, a0);
        a1 = fma(gv.y, zv.y, a1);
    }
    return a0 + a1;
}

// sum_k col[k * cs] * v[k * vs] for k < n with four partial sums and the
// loads unrolled 16 deep (block-inverse columns read from global memory on the
// large elements need many loads in flight)
// Storage of the element block inverses a sweep reads: BF16 for the FP32
// sweep (an approximate inverse only defines the preconditioner, a fixed
// linear operator; the FP32 inner solves take as many iterations with it),
// FP64 for the FP64 sweep.  Entries are widened to T on use.
template <typename T>
struct BlockStore;
template <>
struct BlockStore<float> {
    using type = __nv_bfloat16;
};
template <>
struct BlockStore<double> {
    using type = double;
};
__device__ __forceinline__ float widen(__nv_bfloat16 b) { return __bfloat162float(b); }
__device__ __forceinline__ double widen(double b) { return b; }

// shared-memory units of T an element block of n entries of TB takes
// (16-byte multiples)
template <typename T, typename TB>
__host__ __device__ __forceinline__ int block_units(int n) {
    return (int)((((int64_t)n * (int64_t)sizeof(TB) + 15) / 16) * 16 / (int64_t)sizeof(T));
}

template <typename T, typename TB>
__device__ __forceinline__ T strided_dot(const TB* col, int cs, const T* v, int vs, int n) {
    T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
    int k = 0;
#pragma unroll 4
    for (; k + 4 <= n; k += 4) {
        a0 += widen(col[(k + 0) * cs]) * v[(k + 0) * vs];
        a1 += widen(col[(k + 1) * cs]) * v[(k + 1) * vs];
        a2 += widen(col[(k + 2) * cs]) * v[(k + 2) * vs];
        a3 += widen(col[(k + 3) * cs]) * v[(k + 3) * vs];
    }
    for (; k < n; ++k) a0 += widen(col[k * cs]) * v[k * vs];
    return (a0 + a1) + (a2 + a3);
}

// Stage an element block of n entries with 16-byte copies (its global start
// is 16-byte aligned: block offsets are padded to 8 entries, and the array
// holds 8 entries of padding past its end, so the last copy may run past the
// block).  The destination holds block_units<T, TB>(n) units of T.
template <typename TB>
__device__ __forceinline__ void stage_block(TB* dst, const TB* src, int n) {
    constexpr int kVec = 16 / (int)sizeof(TB);
    const int nv = (n + kVec - 1) / kVec;
    for (int t = threadIdx.x; t < nv; t += blockDim.x) cp_async16(dst + t * kVec, src + t * kVec);
}

template <typename T>
struct UpwindMap {
    int reg_cap = 0;                 // the largest one-phase region (upwind values and map) this launch takes (values)
    int stage_cap = 0;               // values of shared memory after rhs and zpre: a one-phase element whose
                                     // region and block inverse fit stages the inverse too
    const int64_t* up = nullptr;     // upwind value offsets into z
    const typename MapStore<T>::type* G = nullptr;   // maps (this precision's copy)
};

template <typename T>
__global__ void __launch_bounds__(kSweepThreads, 4)
sweep_persistent_kernel(OpView<T> v, const int32_t* __restrict__ rec, int rstride, int ne,
                        const uint8_t* __restrict__ active, const typename BlockStore<T>::type* __restrict__ inv,
                        const T* __restrict__ rin, T* z, unsigned int* __restrict__ next,
                        int* __restrict__ status, UpwindMap<T> um, int rhs_cap, int bcap,
                        unsigned long long* __restrict__ trace) {
    using TB = typename BlockStore<T>::type;
    extern __shared__ __align__(16) unsigned char sraw[];
    T* rhs = reinterpret_cast<T*>(sraw);      // rin, then the couplings c (face nodes)
    T* zpre = rhs + rhs_cap;                  // B rin
    T* Bs = zpre + rhs_cap;
    T* cs = Bs + bcap;   // staged couplings: per active coupling Es | Et | upwind face line | T
    // one-phase path: the upwind values and G_e take the place of Bs and cs
    constexpr uint8_t kOkBit = sizeof(T) == 8 ? 2 : 1;
    constexpr int kP = sizeof(T) == 8 ? 1 : 0;   // this precision's slot among the record's per-precision words
    __shared__ int s_idx;
    __shared__ int s_abort;
    __shared__ int s_rec[kRecMax];
    __shared__ T s_dc[kMaxCplStaged];
    if (v.stop && *v.stop) return;
    for (;;) {
        unsigned long long t_claim = 0;
        if (threadIdx.x == 0) {
            s_idx = (int)atomicAdd(next, 1u);
            s_abort = 0;
            if (trace) t_claim = globaltimer_ns();
        }
        __syncthreads();
        const int idx = s_idx;
        if (idx >= ne) break;
        // the element's record: one coalesced load after the claim
        const int32_t* rp = rec + (int64_t)idx * rstride;
        for (int w = threadIdx.x; w < rstride; w += blockDim.x) s_rec[w] = __ldg(rp + w);
        __syncthreads();
        const int e = s_rec[kRecE];
        if (trace && threadIdx.x == 0) trace[kTr * e] = t_claim;
        if (v.skip && v.skip[s_rec[kRecCol]]) {
            // left out (a converged instance of a batch): no work and no
            // values; only elements left out with it read them
            __syncthreads();
            continue;
        }
        const int nx = s_rec[kRecNx], ny = s_rec[kRecNy], nth = s_rec[kRecNth];
        const int nn = nx * ny, nloc = nn * nth;
        const int bm = s_rec[kRecFlags] >> 4;
        const int64_t dof_off = rec64(s_rec + kRecDof);
        // ---- independent of the sweep: block inverse, residual, mortars
        const TB* B = inv + rec64(s_rec + kRecInv);
        const int bsize = nth * nn * nn;
        if ((s_rec[kRecOk] & kOkBit) && s_rec[kRecReg + kP] <= um.reg_cap) {
            // ---- one-phase path: zpre = B rin and G_e staged before the wait,
            // then z = zpre + G_e z_upwind once the upwind values arrive
            using TG = typename MapStore<T>::type;
            constexpr int kVec = 16 / sizeof(TG);  // map entries per 16-byte copy
            const int nup = s_rec[kRecNup];
            const int ld = map_ld<T>(nup);         // upwind values (T) and map row entries (TG)
            const int gsz = ld * nloc;             // a multiple of kVec
            T* zl = Bs;
            TG* Gs = reinterpret_cast<TG*>(Bs + ld);
            TB* Bg = reinterpret_cast<TB*>(Gs + gsz);
            const TG* Gg = um.G + rec64(s_rec + kRecGoff + 2 * kP);
            const int64_t* up = um.up + rec64(s_rec + kRecUoff);
            for (int t = threadIdx.x; t < gsz / kVec; t += blockDim.x) cp_async16(Gs + t * kVec, Gg + t * kVec);
            // B is read once here (B rin, before the wait): staged with the map
            // when both fit, else read where it lies (coalesced over ij)
            const bool bstaged = s_rec[kRecReg + kP] + block_units<T, TB>(bsize) <= um.stage_cap;
            if (bstaged) stage_block(Bg, B, bsize);
            const TB* Bv = bstaged ? Bg : B;
            for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
                const int ij = l / nth;
                rhs[l] = bdry_node_s(bm, ij / ny, ij % ny, nx, ny) ? T(0) : rin[dof_off + l];
            }
            int64_t my_up = threadIdx.x < nup ? __ldg(up + threadIdx.x) : 0;
            cp_async_wait_all();
            __syncthreads();
            for (int t = threadIdx.x; t < nloc; t += blockDim.x) {
                const int r = t / nn, ij = t % nn;
                zpre[ij * nth + r] = strided_dot(Bv + r * nn * nn + ij, nn, rhs + r, nth, nn);
            }
            long long ck0 = 0, ck1 = 0;
            if (trace && threadIdx.x == 0) {
                trace[kTr * e + 1] = globaltimer_ns();
                ck0 = clock64();
            }
            for (int u = threadIdx.x; u < ld; u += blockDim.x) {
                T val = T(0);
                if (u < nup) {
                    const int64_t o = u == threadIdx.x ? my_up : __ldg(up + u);
                    if (!load_published(z + o, val, status)) s_abort = 1;
                }
                zl[u] = val;   // padding: zero
            }
            __syncthreads();
            if (s_abort) break;
            if (trace && threadIdx.x == 0) ck1 = clock64();
            // FP64 (bound by the FP64 pipe): two threads per output when the
            // CTA has them, the second half of the upwind values through rhs
            // (free once zpre is formed).  FP32 is latency bound and keeps one
            // thread per output (the extra barrier costs more than it saves).
            const bool split = sizeof(T) == 8 && 2 * nloc <= (int)blockDim.x;
            const int nvec = ld / kVec;                 // 16-byte units per row
            const int vh = split ? (nvec + 1) / 2 : nvec;
            T part = T(0);
            const int t = threadIdx.x;
            const int l = split ? t % nloc : t;
            const int half = split ? t / nloc : 0;
            if (!split || t < 2 * nloc) {
                for (int l2 = l; l2 < nloc; l2 += blockDim.x) {
                    const int q0 = half ? vh : 0, q1 = half ? nvec : vh;
                    part = map_row(Gs + (size_t)l2 * ld, zl, q0, q1, half ? T(0) : zpre[l2]);
                    if (half) rhs[l2] = part;
                    else if (!split) st_relaxed(z + dof_off + l2, part);
                }
            }
            if (split) {
                __syncthreads();
                if (t < nloc) st_relaxed(z + dof_off + t, part + rhs[t]);
            }
            __syncthreads();
            if (trace && threadIdx.x == 0) {
                const long long ck4 = clock64();
                trace[kTr * e + 2] = globaltimer_ns();
                trace[kTr * e + 3] = (unsigned long long)blockIdx.x;
                trace[kTr * e + 4] = (unsigned long long)(ck1 - ck0);
                trace[kTr * e + 5] = 0;
                trace[kTr * e + 6] = 0;
                trace[kTr * e + 7] = (unsigned long long)(ck4 - ck1);
            }
            continue;
        }
        const bool staged = block_units<T, TB>(bsize) <= bcap;
        TB* Bsb = reinterpret_cast<TB*>(Bs);
        if (staged) {   // asynchronous copies: every load in flight at once
            stage_block(Bsb, B, bsize);
        } else {
            // too large for shared memory: pull the block into L2 now (one
            // prefetch per 128-byte line, all in flight) for the products below
            const char* b0 = reinterpret_cast<const char*>(B);
            const int64_t nbytes = (int64_t)bsize * sizeof(TB);
            for (int64_t o = (int64_t)threadIdx.x * 128; o < nbytes; o += (int64_t)blockDim.x * 128)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(b0 + o));
        }
        const TB* Bv = staged ? Bsb : B;
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            const int ij = l / nth;
            rhs[l] = bdry_node_s(bm, ij / ny, ij % ny, nx, ny) ? T(0) : rin[dof_off + l];
        }
        // the active couplings (in coupling order) and the face nodes they
        // reach, from the record; their mortars staged with asynchronous
        // copies, waited on with the block inverse's
        const int ncs = s_rec[kRecNcs], nf = s_rec[kRecNf];
        const int* s_cpl = s_rec + kRecHead;
        const int* s_face = s_cpl + kRecCpl * max(ncs, 0);
        for (int c = 0; c < ncs; ++c) {
            const int* cp = s_cpl + kRecCpl * c;
            const int m1 = cp[kCplM1], n0 = cp[kCplN0], nt1 = cp[kCplNt1];
            T* dst = cs + cp[kCplOff];
            const T* es = v.mort + cp[kCplEs];
            const T* et = v.mort + cp[kCplEt];
            for (int t = threadIdx.x; t < m1 * n0; t += blockDim.x) cp_async_small<sizeof(T)>(dst + t, es + t);
            for (int t = threadIdx.x; t < nt1 * nth; t += blockDim.x)
                cp_async_small<sizeof(T)>(dst + m1 * n0 + t, et + t);
        }
        if ((int)threadIdx.x < ncs) s_dc[threadIdx.x] = v.cplc[s_cpl[kRecCpl * threadIdx.x + kCplK]];
        cp_async_wait_all();
        __syncthreads();
        // zpre = B rin, block stored as [r][k][ij]
        for (int t = threadIdx.x; t < nloc; t += blockDim.x) {
            const int r = t / nn, ij = t % nn;
            zpre[ij * nth + r] = strided_dot(Bv + r * nn * nn + ij, nn, rhs + r, nth, nn);
        }
        // ---- couplings c on the face nodes, into rhs[ij * nth + r]
        long long ck0 = 0, ck1 = 0, ck2 = 0, ck3 = 0;   // phase clocks (thread 0, traced sweeps)
        if (trace && threadIdx.x == 0) {
            trace[kTr * e + 1] = globaltimer_ns();
            ck0 = clock64();
        }
        if (ncs > 0 && s_rec[kRecDirect]) {
            // diagonal mortars: c on the face nodes straight from the upwind
            // values, c[q][r] = sum_couplings dcoeff Es[q][q] Et[r][r] z_up[q][r]
            // (each thread waits on its own values); no T, no mortar sums.
            // The couplings overwrite rin at the face nodes: B rin is formed first.
            __syncthreads();
            for (int t = threadIdx.x; t < nf * nth; t += blockDim.x) {
                const int ij = s_face[t / nth], r = t % nth, i = ij / ny, j = ij % ny;
                T acc = T(0);
                for (int c = 0; c < ncs; ++c) {
                    const int* cp = s_cpl + kRecCpl * c;
                    const int F = cp[kCplF];
                    if (!on_face(F, i, j, nx, ny)) continue;
                    const int q = (F % 2 == 0) ? j : i;
                    const int n0 = cp[kCplN0];
                    const T* Es = cs + cp[kCplOff];
                    const T* Et = Es + cp[kCplM1] * n0;
                    T val = T(0);
                    if (!load_published(z + rec64(cp + kCplBase) + (int64_t)q * cp[kCplStr] + r, val, status))
                        s_abort = 1;
                    acc += s_dc[c] * (Es[q * n0 + q] * (Et[r * nth + r] * val));
                }
                rhs[ij * nth + r] = acc;
            }
        } else if (ncs >= 0) {
            // stage the upwind face lines as they are published (coalesced,
            // each value once; each thread waits on its own values)
            for (int c = 0; c < ncs; ++c) {
                const int* cp = s_cpl + kRecCpl * c;
                const int m1 = cp[kCplM1], nt1 = cp[kCplNt1];
                T* dst = cs + cp[kCplOff] + m1 * cp[kCplN0] + nt1 * nth;
                const T* src = z + rec64(cp + kCplBase);
                const int str = cp[kCplStr];
                for (int t = threadIdx.x; t < m1 * nt1; t += blockDim.x) {
                    const int jj = t / nt1, a = t % nt1;
                    T val = T(0);
                    if (!load_published(src + (int64_t)jj * str + a, val, status)) s_abort = 1;
                    dst[t] = val;
                }
            }
            __syncthreads();
            if (s_abort) break;
            if (trace && threadIdx.x == 0) ck1 = clock64();
            // T[jj][r] = sum_a Et[a][r] zl[jj][a], all couplings at once
            {
                int c = 0, base = 0;
                for (int t = threadIdx.x;; t += blockDim.x) {
                    // advance to the coupling that holds item t
                    while (c < ncs && t >= base + s_cpl[kRecCpl * c + kCplM1] * nth) {
                        base += s_cpl[kRecCpl * c + kCplM1] * nth;
                        ++c;
                    }
                    if (c >= ncs) break;
                    const int* cp = s_cpl + kRecCpl * c;
                    const int dg = cp[kCplDiag];
                    if (dg == 3) continue;   // Es and Et diagonal: the face phase reads the line itself
                    const int m1 = cp[kCplM1], nt1 = cp[kCplNt1];
                    const T* Et = cs + cp[kCplOff] + m1 * cp[kCplN0];
                    const T* zl = Et + nt1 * nth;
                    T* Tm = cs + cp[kCplOff] + m1 * cp[kCplN0] + nt1 * nth + m1 * nt1;
                    const int q = t - base, jj = q / nth, r = q % nth;
                    T acc = T(0);
                    if (dg & 2) {
                        acc = Et[r * nth + r] * zl[jj * nt1 + r];
                    } else {
                        for (int a = 0; a < nt1; ++a) acc += Et[a * nth + r] * zl[jj * nt1 + a];
                    }
                    Tm[jj * nth + r] = acc;
                }
            }
            __syncthreads();
            if (trace && threadIdx.x == 0) ck2 = clock64();
            for (int t = threadIdx.x; t < nf * nth; t += blockDim.x) {
                const int ij = s_face[t / nth], r = t % nth, i = ij / ny, j = ij % ny;
                T acc = T(0);
                for (int c = 0; c < ncs; ++c) {
                    const int* cp = s_cpl + kRecCpl * c;
                    const int F = cp[kCplF];
                    if (!on_face(F, i, j, nx, ny)) continue;
                    const int m1 = cp[kCplM1], n0 = cp[kCplN0], nt1 = cp[kCplNt1], dg = cp[kCplDiag];
                    const int qq = (F % 2 == 0) ? j : i;
                    const T* Es = cs + cp[kCplOff];
                    const T* Et = Es + m1 * n0;
                    const T* zl = Et + nt1 * nth;
                    const T* Tm = zl + m1 * nt1;
                    T sacc = T(0);
                    if (dg == 3) {
                        sacc = Es[qq * n0 + qq] * (Et[r * nth + r] * zl[qq * nt1 + r]);
                    } else if (dg & 1) {
                        sacc = Es[qq * n0 + qq] * Tm[qq * nth + r];
                    } else {
                        for (int jj = 0; jj < m1; ++jj) sacc += Es[jj * n0 + qq] * Tm[jj * nth + r];
                    }
                    acc += s_dc[c] * sacc;
                }
                rhs[ij * nth + r] = acc;
            }
        } else {
            for (int t = threadIdx.x; t < nf * nth; t += blockDim.x) {
                const int ij = s_face[t / nth], r = t % nth, i = ij / ny, j = ij % ny;
                T acc = T(0);
                for (int k = s_rec[kRecCplB]; k < s_rec[kRecCplE]; ++k) {
                    if (!active[k]) continue;
                    const CplDev cp = v.cpls[k];
                    const int F = cp.face;
                    if (!on_face(F, i, j, nx, ny)) continue;
                    const CplGeo g = v.cgeo[k];
                    const int qq = (F % 2 == 0) ? j : i;
                    const int n0 = (F % 2 == 0) ? ny : nx;
                    const T* Es = v.mort + cp.es;
                    const T* Et = v.mort + cp.et;
                    const T dc = v.cplc[k];
                    for (int jj = 0; jj < g.m1; ++jj) {
                        const T* zl = z + g.base + (int64_t)jj * g.stride;
                        T sacc = T(0);
                        for (int a = 0; a < g.nth1; ++a) {
                            T val = T(0);
                            if (!load_published(zl + a, val, status)) s_abort = 1;
                            sacc += Et[a * nth + r] * val;
                        }
                        acc += dc * Es[jj * n0 + qq] * sacc;
                    }
                }
                rhs[ij * nth + r] = acc;
            }
        }
        __syncthreads();
        if (s_abort) break;
        if (trace && threadIdx.x == 0) ck3 = clock64();
        // ---- z = zpre - B c over the face columns of B
        for (int t = threadIdx.x; t < nloc; t += blockDim.x) {
            const int r = t / nn, ij = t % nn;
            const TB* col = Bv + r * nn * nn + ij;
            T a0 = zpre[ij * nth + r], a1 = T(0), a2 = T(0), a3 = T(0);
            int f = 0;
#pragma unroll 2
            for (; f + 4 <= nf; f += 4) {
                a0 -= widen(col[s_face[f + 0] * nn]) * rhs[s_face[f + 0] * nth + r];
                a1 -= widen(col[s_face[f + 1] * nn]) * rhs[s_face[f + 1] * nth + r];
                a2 -= widen(col[s_face[f + 2] * nn]) * rhs[s_face[f + 2] * nth + r];
                a3 -= widen(col[s_face[f + 3] * nn]) * rhs[s_face[f + 3] * nth + r];
            }
            for (; f < nf; ++f) a0 -= widen(col[s_face[f] * nn]) * rhs[s_face[f] * nth + r];
            st_relaxed(z + dof_off + (int64_t)ij * nth + r, (a0 + a1) + (a2 + a3));
        }
        // the stored values are the publication (downstream elements wait on
        // the values themselves); the barrier ends this element's use of the
        // shared buffers before the next claim
        __syncthreads();
        if (trace && threadIdx.x == 0) {
            const long long ck4 = clock64();
            trace[kTr * e + 2] = globaltimer_ns();
            trace[kTr * e + 3] = (unsigned long long)blockIdx.x;
            // SM clock cycles of the phases after the independent work
            // (staged path; on the other path the first two stay 0)
            trace[kTr * e + 4] = (unsigned long long)(ck1 ? ck1 - ck0 : 0);
            trace[kTr * e + 5] = (unsigned long long)(ck2 ? ck2 - ck1 : 0);
            trace[kTr * e + 6] = (unsigned long long)(ck3 - (ck2 ? ck2 : ck0));
            trace[kTr * e + 7] = (unsigned long long)(ck4 - ck3);
        }
    }
}

// BF16 copy of the FP32 block inverses (round to nearest even), the FP32 sweep's
__global__ void to_bf16_kernel(const float* __restrict__ in, __nv_bfloat16* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

// Builds the upwind maps G_e = -B_e C_e of the one-phase elements in FP64
// (and the FP32 sweep's BF16 copies, rounded to nearest even; rows of map_ld
// entries, padding left zero): entry
// (u, l) with u = (coupling k, jj, a) and l = (ij, r) is -dcoeff_k Et_k[a][r] sum_q B_r[ij][f_q] Es_k[jj][q] over the
// nodes f_q of coupling k's face that are not inflow-boundary nodes.  One CTA
// per element.
__global__ void build_upwind_map_kernel(OpView<double> v, const uint8_t* __restrict__ active,
                                        const double* __restrict__ inv, const int64_t* __restrict__ inv_elem_off,
                                        const int32_t* __restrict__ elems, const int32_t* __restrict__ nup_e,
                                        const int64_t* __restrict__ goff64, const int64_t* __restrict__ goff32,
                                        double* __restrict__ G64, __nv_bfloat16* __restrict__ G16) {
    const int e = elems[blockIdx.x];
    const ElemDev E = v.elems[e];
    const ColDev C = v.cols[E.col];
    const int nth = E.nth, nn = C.nx * C.ny, nloc = nn * nth, bm = E.flags >> 4;
    const int nup = nup_e[e];
    const double* B = inv + inv_elem_off[e];
    for (int t = threadIdx.x; t < nup * nloc; t += blockDim.x) {
        const int u = t / nloc, l = t % nloc, ij = l / nth, r = l % nth;
        int uu = u, k = E.cpl_begin;
        for (; k < E.cpl_end; ++k) {
            if (!active[k]) continue;
            const int sz = v.cgeo[k].m1 * v.cgeo[k].nth1;
            if (uu < sz) break;
            uu -= sz;
        }
        const CplGeo g = v.cgeo[k];
        const CplDev cp = v.cpls[k];
        const int jj = uu / g.nth1, a = uu % g.nth1;
        const int F = cp.face;
        const int n0 = (F % 2 == 0) ? C.ny : C.nx;
        const double et = v.mort[cp.et + a * nth + r];
        double acc = 0.;
        for (int q = 0; q < n0; ++q) {
            const int i = (F == 0) ? C.nx - 1 : (F == 2) ? 0 : q;
            const int j = (F == 1) ? C.ny - 1 : (F == 3) ? 0 : q;
            if (bdry_node_s(bm, i, j, C.nx, C.ny)) continue;
            acc += B[(int64_t)r * nn * nn + (int64_t)(i * C.ny + j) * nn + ij] * v.mort[cp.es + jj * n0 + q];
        }
        const double val = -v.cplc[k] * et * acc;
        G64[goff64[e] + (int64_t)l * map_ld<double>(nup) + u] = val;
        G16[goff32[e] + (int64_t)l * map_ld<float>(nup) + u] = __float2bfloat16_rn((float)val);
    }
}


}  // namespace

struct Sweep {
    int nlev = 0;
    std::vector<int32_t> lev_start;      // host CSR over levels
    std::vector<int32_t> h_lev_elems;    // elements in level order (host copy)
    int32_t* d_lev_elems = nullptr;
    uint8_t* d_active = nullptr;
    double* d_inv64 = nullptr;
    float* d_inv32 = nullptr;
    __nv_bfloat16* d_inv16 = nullptr;   // the FP32 sweep's copy
    int64_t* d_inv_off = nullptr;
    int64_t inv_entries = 0;
    int max_nloc = 0;
    int64_t max_b = 0, max_c = 0;
    // launch shapes per precision (0 FP32, 1 FP64): kSweepShapes shared-memory
    // budgets, the fastest chosen by timing the first sweep of the handle
    struct Shape {
        size_t smem = 0;
        int bcap = 0, grid = 0, reg_cap = 0, threads = kSweepThreads;
    };
    Shape shape[2][kSweepShapes];
    int pick[2] = {-1, -1};
    float shape_ms[2][kSweepShapes] = {};
    int32_t *d_greg32 = nullptr, *d_greg64 = nullptr;
    int32_t* d_rec = nullptr;            // element records in claim order
    int rec_stride = 0;                  // words per record (a multiple of 32)
    int n_lagged = 0;
    std::vector<void*> allocs;
    unsigned int* d_next = nullptr;      // work counter
    int* d_status = nullptr;             // RTG_ERR_TIMEOUT if a wait gave up
    // one-phase elements (upwind maps)
    uint8_t* d_gok = nullptr;
    int32_t* d_gnup = nullptr;
    int64_t *d_goff64 = nullptr, *d_goff32 = nullptr, *d_uoff = nullptr, *d_up = nullptr;
    double* d_G64 = nullptr;
    __nv_bfloat16* d_G16 = nullptr;     // the FP32 sweep's copy
    int64_t gmax32 = 0, gmax64 = 0;     // largest one-phase region with its block inverse (values) per precision
    int64_t g_entries = 0;
    // per precision (FP32, FP64), the elements with a map: the region the map
    // and the upwind values take (values), map entries, upwind indices; a
    // launch shape uses the maps whose region fits it
    struct MapUse {
        int64_t region, entries, nup;
    };
    std::vector<MapUse> onephase[2];
};

namespace {

template <typename T>
T* sw_alloc(Sweep* s, size_t n) {
    void* p = nullptr;
    RTG_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)));
    s->allocs.push_back(p);
    return (T*)p;
}

}  // namespace

void free_sweep(rtg_handle* h) {
    Sweep* s = h->sweep;
    if (!s) return;
    for (void* p : s->allocs) cudaFree(p);
    delete s;
    h->sweep = nullptr;
}

Sweep* get_sweep(rtg_handle* h, cudaStream_t st) {
    if (h->sweep) return h->sweep;
    const HostTables& t = h->host;
    const int ne = (int)t.elems.size();
    for (const ColDev& C : t.cols)
        if (C.nx * C.ny > kMaxBlock)
            throw RtgError{RTG_ERR_SIZE, "sweep preconditioner supports nx*ny <= 100"};
    Sweep* s = new Sweep();
    h->sweep = s;
    // ---- upwind order: Kahn levels with cycle breaking
    std::vector<std::vector<int32_t>> succ(ne);
    std::vector<int32_t> indeg(ne, 0);
    for (int e = 0; e < ne; ++e)
        for (int k = t.elems[e].cpl_begin; k < t.elems[e].cpl_end; ++k) {
            const int p = t.cpls[k].nbr;
            if (p == e) continue;
            succ[p].push_back(e);
            indeg[e]++;
        }
    // Kahn's algorithm, ready elements taken lowest level first; a cycle is
    // broken by forcing the lowest-index unprocessed element.
    std::vector<int32_t> level(ne, -1);
    std::vector<char> done(ne, 0);
    std::vector<int32_t> order;
    order.reserve(ne);
    std::priority_queue<std::pair<int, int>, std::vector<std::pair<int, int>>, std::greater<>> ready;
    std::vector<int32_t> lvl_pred(ne, 0);  // 1 + max level of processed predecessors
    for (int e = 0; e < ne; ++e)
        if (indeg[e] == 0) ready.push({0, e});
    int processed = 0;
    int next_forced = 0;
    while (processed < ne) {
        if (ready.empty()) {
            // cycle: force the lowest-index unprocessed element
            while (next_forced < ne && done[next_forced]) ++next_forced;
            const int e = next_forced;
            s->n_lagged += indeg[e];
            indeg[e] = 0;
            ready.push({lvl_pred[e], e});
        }
        const auto top = ready.top();
        ready.pop();
        const int e = top.second;
        if (done[e]) continue;
        done[e] = 1;
        level[e] = lvl_pred[e];
        order.push_back(e);
        ++processed;
        for (int q : succ[e]) {
            if (done[q]) continue;
            lvl_pred[q] = std::max(lvl_pred[q], level[e] + 1);
            if (--indeg[q] == 0) ready.push({lvl_pred[q], q});
        }
    }
    int nlev = 0;
    for (int e = 0; e < ne; ++e) nlev = std::max(nlev, level[e] + 1);
    s->nlev = nlev;
    s->lev_start.assign(nlev + 1, 0);
    for (int e = 0; e < ne; ++e) s->lev_start[level[e] + 1]++;
    for (int L = 0; L < nlev; ++L) s->lev_start[L + 1] += s->lev_start[L];
    std::vector<int32_t> lev_elems(ne), fill(s->lev_start.begin(), s->lev_start.end() - 1);
    for (int e = 0; e < ne; ++e) lev_elems[fill[level[e]]++] = e;
    // within a level, the elements with the longest chain of levels below
    // them first (list scheduling by bottom level), then by index: the CTAs
    // claim the critical chains early (any order within a level is a valid
    // claim order, every predecessor sits on an earlier level)
    {
        std::vector<int32_t> blev(ne, 0);
        for (int L = nlev - 1; L >= 0; --L)
            for (int q = s->lev_start[L]; q < s->lev_start[L + 1]; ++q) {
                const int e = lev_elems[q];
                int b = 0;
                for (int d : succ[e])
                    if (level[d] > level[e]) b = std::max(b, blev[d] + 1);
                blev[e] = b;
            }
        for (int L = 0; L < nlev; ++L)
            std::stable_sort(lev_elems.begin() + s->lev_start[L], lev_elems.begin() + s->lev_start[L + 1],
                             [&](int x, int y) { return blev[x] > blev[y]; });
    }
    s->h_lev_elems = lev_elems;
    // a coupling is active when its upwind element sits on an earlier level
    std::vector<uint8_t> active(t.cpls.size(), 0);
    for (int e = 0; e < ne; ++e)
        for (int k = t.elems[e].cpl_begin; k < t.elems[e].cpl_end; ++k)
            active[k] = level[t.cpls[k].nbr] < level[e] ? 1 : 0;
    // ---- element block inverses.  An element's blocks are a function of its
    // node counts, face and boundary flags, extinction and streaming constants,
    // angular table and the column's wx wy kappa values (what
    // build_block_inverse_kernel reads); elements that agree on the bits of
    // all of them share one copy (the sweep reaches blocks through
    // inv_elem_off), so they are built and stored once.
    std::vector<int32_t> blk_elem, blk_r;
    std::vector<int64_t> blk_off, inv_off(ne);
    int64_t off = 0, entries = 0;
    int max_nn = 1;
    std::unordered_map<std::vector<uint64_t>, int64_t, WordsHash> shared;
    shared.reserve((size_t)ne);
    auto bits = [](double x) {
        uint64_t u;
        std::memcpy(&u, &x, sizeof(u));
        return u;
    };
    for (int e = 0; e < ne; ++e) {
        const ElemDev& E = t.elems[e];
        const ColDev& C = t.cols[E.col];
        const int nn = C.nx * C.ny;
        max_nn = std::max(max_nn, nn);
        s->max_nloc = std::max(s->max_nloc, nn * E.nth);
        entries += (int64_t)E.nth * nn * nn;
        std::vector<uint64_t> key = {(uint64_t)C.nx, (uint64_t)C.ny, (uint64_t)E.nth, (uint64_t)E.flags};
        for (int q = 0; q < 3; ++q) key.push_back(bits(t.econst[4 * (size_t)e + q]));
        for (int q = 0; q < 7 * E.nth; ++q) key.push_back(bits(t.ang[(size_t)E.ang + q]));
        for (int q = 0; q < nn; ++q) key.push_back(bits(t.kw[(size_t)C.node_off + q]));
        auto hit = shared.find(key);
        if (hit != shared.end()) {
            inv_off[e] = hit->second;
            continue;
        }
        // each distinct block set starts on 8 values (16 bytes in BF16), so
        // that the sweep stages it with 16-byte copies
        off = (off + 7) & ~int64_t(7);
        inv_off[e] = off;
        shared.emplace(std::move(key), off);
        for (int r = 0; r < E.nth; ++r) {
            blk_elem.push_back(e);
            blk_r.push_back(r);
            blk_off.push_back(off);
            off += (int64_t)nn * nn;
        }
    }
    s->inv_entries = entries;   // algorithmic entries (the padding excluded)
    s->d_lev_elems = sw_alloc<int32_t>(s, ne);
    s->d_active = sw_alloc<uint8_t>(s, active.size());
    s->d_inv_off = sw_alloc<int64_t>(s, ne);
    // 8 entries of padding past the last block: a staging copy may run past
    // the end of its block
    s->d_inv64 = sw_alloc<double>(s, off + 8);
    s->d_inv32 = sw_alloc<float>(s, off + 8);
    s->d_inv16 = sw_alloc<__nv_bfloat16>(s, off + 8);
    RTG_CUDA(cudaMemsetAsync(s->d_inv64, 0, sizeof(double) * (size_t)(off + 8), st));
    RTG_CUDA(cudaMemsetAsync(s->d_inv32, 0, sizeof(float) * (size_t)(off + 8), st));
    int32_t* d_be = sw_alloc<int32_t>(s, blk_elem.size());
    int32_t* d_br = sw_alloc<int32_t>(s, blk_r.size());
    int64_t* d_bo = sw_alloc<int64_t>(s, blk_off.size());
    int* d_status = sw_alloc<int>(s, 1);
    RTG_CUDA(cudaMemcpy(s->d_lev_elems, lev_elems.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice));
    if (!active.empty())
        RTG_CUDA(cudaMemcpy(s->d_active, active.data(), active.size(), cudaMemcpyHostToDevice));
    RTG_CUDA(cudaMemcpy(s->d_inv_off, inv_off.data(), sizeof(int64_t) * ne, cudaMemcpyHostToDevice));
    RTG_CUDA(cudaMemcpy(d_be, blk_elem.data(), sizeof(int32_t) * blk_elem.size(), cudaMemcpyHostToDevice));
    RTG_CUDA(cudaMemcpy(d_br, blk_r.data(), sizeof(int32_t) * blk_r.size(), cudaMemcpyHostToDevice));
    RTG_CUDA(cudaMemcpy(d_bo, blk_off.data(), sizeof(int64_t) * blk_off.size(), cudaMemcpyHostToDevice));
    RTG_CUDA(cudaMemset(d_status, 0, sizeof(int)));
    const size_t smem = sizeof(float) * (size_t)max_nn * 2 * max_nn;
    raise_smem_limit((const void*)build_block_inverse_kernel, smem);
    build_block_inverse_kernel<<<(int)blk_elem.size(), 256, smem, st>>>(h->v32, d_be, d_br, d_bo, s->d_inv64,
                                                                         s->d_inv32, d_status), count_launch();
    RTG_CUDA(cudaGetLastError());
    int status = 0;
    RTG_CUDA(cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    RTG_CUDA(cudaStreamSynchronize(st));
    if (status) throw RtgError{RTG_ERR_NONFINITE, "singular element block in the sweep preconditioner"};
    to_bf16_kernel<<<std::max<int64_t>(1, std::min<int64_t>((off + 8 + 255) / 256, 152 * 8)), 256, 0, st>>>(
        s->d_inv32, s->d_inv16, off + 8), count_launch();
    RTG_CUDA(cudaGetLastError());
    s->d_next = sw_alloc<unsigned int>(s, 1);
    s->d_status = sw_alloc<int>(s, 1);
    RTG_CUDA(cudaMemset(s->d_status, 0, sizeof(int)));
    int64_t max_b = 0;
    for (int e = 0; e < ne; ++e) {
        const ColDev& C = t.cols[t.elems[e].col];
        max_b = std::max<int64_t>(max_b, (int64_t)t.elems[e].nth * C.nx * C.ny * C.nx * C.ny);
    }
    s->max_b = max_b;
    int64_t max_c = 0;
    for (int e = 0; e < ne; ++e) {
        const ElemDev& E = t.elems[e];
        const ColDev& C = t.cols[E.col];
        int64_t c = 0;
        for (int k = E.cpl_begin; k < E.cpl_end; ++k) {
            if (!active[k]) continue;
            const CplGeo& g = t.cgeo[k];
            const int n0 = (t.cpls[k].face % 2 == 0) ? C.ny : C.nx;
            c += (int64_t)g.m1 * n0 + (int64_t)g.nth1 * E.nth + (int64_t)g.m1 * g.nth1 + (int64_t)g.m1 * E.nth;
        }
        max_c = std::max(max_c, c);
    }
    s->max_c = max_c;
    // ---- upwind maps of the elements whose map fits in shared memory.  A map
    // is a function of the element's (shared) block inverses and of its active
    // couplings' faces, sizes, mortars and dcoeff; elements that agree on them
    // share one stored map (built once, by the first of them).
    {
        const int rhs_cap = (std::max(s->max_nloc, 1) + 1) & ~1;   // even: 16-byte aligned region after rhs, zpre
        std::vector<uint8_t> gok(ne, 0);
        std::vector<int32_t> gnup(ne, 0), gel, greg32(ne, 0), greg64(ne, 0);
        std::vector<int64_t> goff64(ne, 0), goff32(ne, 0), uoff(ne, 0), up;
        int64_t gtot64 = 0, gtot32 = 0;
        std::unordered_map<std::vector<uint64_t>, std::pair<int64_t, int64_t>, WordsHash> gshared;
        gshared.reserve((size_t)ne);
        for (int e = 0; e < ne; ++e) {
            const ElemDev& E = t.elems[e];
            const ColDev& C = t.cols[E.col];
            const int nloc = C.nx * C.ny * E.nth;
            int64_t nup = 0;
            for (int k = E.cpl_begin; k < E.cpl_end; ++k)
                if (active[k]) nup += (int64_t)t.cgeo[k].m1 * t.cgeo[k].nth1;
            // upwind values (one map row long), G_e, then B_e
            const int64_t bsize = (int64_t)E.nth * C.nx * C.ny * C.nx * C.ny;
            const int64_t ld32 = map_ld<float>((int)nup), ld64 = map_ld<double>((int)nup);
            // FP32 sweep: upwind values in FP32, G_e in BF16 (ld32 is a multiple
            // of 8, so the map is a whole number of FP32 values); B_e (read
            // once, before the wait) joins them in shared memory when it fits
            const int64_t region32 = ld32 + ld32 * nloc / 2;
            const int64_t region64 = ld64 + ld64 * nloc;
            const int64_t with_b32 = region32 + block_units<float, __nv_bfloat16>((int)bsize);
            const int64_t with_b64 = region64 + block_units<double, double>((int)bsize);
            uint8_t ok = 0;
            if (region32 * 4 + 2 * rhs_cap * 4 <= (int64_t)kSweepSmemBudget) ok |= 1;
            if (region64 * 8 + 2 * rhs_cap * 8 <= (int64_t)kSweepSmemBudget) ok |= 2;
            if (!ok) continue;
            gok[e] = ok;
            gnup[e] = (int32_t)nup;
            greg32[e] = (int32_t)region32;
            greg64[e] = (int32_t)region64;
            uoff[e] = (int64_t)up.size();
            std::vector<uint64_t> gkey = {(uint64_t)inv_off[e], (uint64_t)E.nth, (uint64_t)E.flags};
            for (int k = E.cpl_begin; k < E.cpl_end; ++k) {
                if (!active[k]) continue;
                const CplGeo& g = t.cgeo[k];
                const CplDev& cp = t.cpls[k];
                gkey.insert(gkey.end(), {(uint64_t)cp.face, (uint64_t)g.m1, (uint64_t)g.nth1, (uint64_t)cp.es,
                                         (uint64_t)cp.et, bits(t.cplc[k])});
            }
            auto ghit = gshared.find(gkey);
            const bool built = ghit == gshared.end();
            if (built) {
                goff64[e] = gtot64;
                goff32[e] = gtot32;
                gshared.emplace(std::move(gkey), std::make_pair(gtot64, gtot32));
                gtot64 += ld64 * nloc;
                gtot32 += ld32 * nloc;
            } else {
                goff64[e] = ghit->second.first;
                goff32[e] = ghit->second.second;
            }
            for (int k = E.cpl_begin; k < E.cpl_end; ++k) {
                if (!active[k]) continue;
                const CplGeo& g = t.cgeo[k];
                for (int jj = 0; jj < g.m1; ++jj)
                    for (int a = 0; a < g.nth1; ++a) up.push_back(g.base + (int64_t)jj * g.stride + a);
            }
            if (ok & 1) s->gmax32 = std::max(s->gmax32, with_b32);
            if (ok & 2) s->gmax64 = std::max(s->gmax64, with_b64);
            for (int p = 0; p < 2; ++p)
                if (ok & (1 << p)) s->onephase[p].push_back({p ? region64 : region32, (p ? ld64 : ld32) * nloc, nup});
            if (built) gel.push_back(e);
        }
        s->g_entries = gtot64 + gtot32;
        s->d_gok = sw_alloc<uint8_t>(s, ne);
        s->d_greg32 = sw_alloc<int32_t>(s, ne);
        s->d_greg64 = sw_alloc<int32_t>(s, ne);
        RTG_CUDA(cudaMemcpy(s->d_greg32, greg32.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemcpy(s->d_greg64, greg64.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice));
        s->d_gnup = sw_alloc<int32_t>(s, ne);
        s->d_goff64 = sw_alloc<int64_t>(s, ne);
        s->d_goff32 = sw_alloc<int64_t>(s, ne);
        s->d_uoff = sw_alloc<int64_t>(s, ne);
        s->d_up = sw_alloc<int64_t>(s, up.size());
        s->d_G64 = sw_alloc<double>(s, gtot64);
        s->d_G16 = sw_alloc<__nv_bfloat16>(s, gtot32);
        RTG_CUDA(cudaMemset(s->d_G64, 0, sizeof(double) * std::max<int64_t>(gtot64, 1)));
        RTG_CUDA(cudaMemset(s->d_G16, 0, sizeof(__nv_bfloat16) * std::max<int64_t>(gtot32, 1)));
        int32_t* d_gel = sw_alloc<int32_t>(s, gel.size());
        RTG_CUDA(cudaMemcpy(s->d_gok, gok.data(), ne, cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemcpy(s->d_gnup, gnup.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemcpy(s->d_goff64, goff64.data(), sizeof(int64_t) * ne, cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemcpy(s->d_goff32, goff32.data(), sizeof(int64_t) * ne, cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemcpy(s->d_uoff, uoff.data(), sizeof(int64_t) * ne, cudaMemcpyHostToDevice));
        if (!up.empty())
            RTG_CUDA(cudaMemcpy(s->d_up, up.data(), sizeof(int64_t) * up.size(), cudaMemcpyHostToDevice));
        if (!gel.empty()) {
            RTG_CUDA(cudaMemcpy(d_gel, gel.data(), sizeof(int32_t) * gel.size(), cudaMemcpyHostToDevice));
            build_upwind_map_kernel<<<(int)gel.size(), 256, 0, st>>>(h->v64, s->d_active, s->d_inv64, s->d_inv_off,
                                                                    d_gel, s->d_gnup, s->d_goff64, s->d_goff32, s->d_G64,
                                                                    s->d_G16), count_launch();
            RTG_CUDA(cudaGetLastError());
        }
        // ---- element records in claim order (the words are listed with kRecE)
        auto bdry = [](int bm, int i, int j, int nx, int ny) {
            return ((bm & 1) && i == nx - 1) || ((bm & 2) && j == ny - 1) || ((bm & 4) && i == 0) ||
                   ((bm & 8) && j == 0);
        };
        auto onf = [](int F, int i, int j, int nx, int ny) {
            return (F == 0 && i == nx - 1) || (F == 1 && j == ny - 1) || (F == 2 && i == 0) || (F == 3 && j == 0);
        };
        auto put64 = [](int32_t* w, int64_t x) {
            w[0] = (int32_t)(uint32_t)((uint64_t)x & 0xFFFFFFFFu);
            w[1] = (int32_t)(uint32_t)((uint64_t)x >> 32);
        };
        std::vector<std::vector<int32_t>> recs(ne);
        size_t rmax = kRecHead;
        for (int idx = 0; idx < ne; ++idx) {
            const int e = lev_elems[idx];
            const ElemDev& E = t.elems[e];
            const ColDev& C = t.cols[E.col];
            std::vector<int32_t>& R = recs[idx];
            R.assign(kRecHead, 0);
            R[kRecE] = e;
            R[kRecCol] = E.col;
            put64(&R[kRecDof], E.dof_off);
            R[kRecNx] = C.nx;
            R[kRecNy] = C.ny;
            R[kRecNth] = E.nth;
            R[kRecFlags] = E.flags;
            put64(&R[kRecInv], inv_off[e]);
            R[kRecCplB] = E.cpl_begin;
            R[kRecCplE] = E.cpl_end;
            R[kRecOk] = gok[e];
            R[kRecReg] = greg32[e];
            R[kRecReg + 1] = greg64[e];
            R[kRecNup] = gnup[e];
            put64(&R[kRecGoff], goff32[e]);
            put64(&R[kRecGoff + 2], goff64[e]);
            put64(&R[kRecUoff], uoff[e]);
            std::vector<int> act;
            int fm = 0;
            for (int k = E.cpl_begin; k < E.cpl_end; ++k)
                if (active[k]) {
                    act.push_back(k);
                    fm |= 1 << t.cpls[k].face;
                }
            const int ncs = (int)act.size() <= kMaxCplStaged ? (int)act.size() : -1;
            R[kRecNcs] = ncs;
            // diagonal mortars (conforming neighbours: the off-diagonal
            // entries are rounding noise, below 1e-13 of the largest, and the
            // preconditioner leaves them out): the face value (q, r) takes only
            // the upwind value (q, r), so the couplings need no T and no sums
            bool direct = ncs > 0;
            auto diagonal = [&](int64_t off, int rows, int cols) {
                double mx = 0.;
                for (int q = 0; q < rows * cols; ++q) mx = std::max(mx, std::fabs(t.mort[(size_t)off + q]));
                for (int a = 0; a < rows; ++a)
                    for (int b = 0; b < cols; ++b)
                        if (a != b && std::fabs(t.mort[(size_t)off + (size_t)a * cols + b]) > 1e-13 * mx) return false;
                return mx > 0.;
            };
            for (int c = 0; c < ncs && direct; ++c) {
                const int k = act[c];
                const CplDev& cp = t.cpls[k];
                const CplGeo& g = t.cgeo[k];
                const int n0 = (cp.face % 2 == 0) ? C.ny : C.nx;
                direct = g.m1 == n0 && g.nth1 == E.nth && diagonal(cp.es, g.m1, n0) && diagonal(cp.et, g.nth1, E.nth);
            }
            R[kRecDirect] = direct ? 1 : 0;
            int soff = 0;
            for (int c = 0; c < ncs; ++c) {
                const int k = act[c];
                const CplDev& cp = t.cpls[k];
                const CplGeo& g = t.cgeo[k];
                const int n0 = (cp.face % 2 == 0) ? C.ny : C.nx;
                int32_t w[kRecCpl] = {};
                w[kCplF] = cp.face;
                w[kCplM1] = g.m1;
                w[kCplNt1] = g.nth1;
                w[kCplN0] = n0;
                w[kCplStr] = g.stride;
                w[kCplEs] = cp.es;
                w[kCplEt] = cp.et;
                put64(&w[kCplBase], g.base);
                w[kCplOff] = soff;
                w[kCplK] = k;
                w[kCplDiag] = (g.m1 == n0 && diagonal(cp.es, g.m1, n0) ? 1 : 0) |
                              (g.nth1 == E.nth && diagonal(cp.et, g.nth1, E.nth) ? 2 : 0);
                R.insert(R.end(), w, w + kRecCpl);
                soff += g.m1 * n0 + g.nth1 * E.nth + g.m1 * g.nth1 + g.m1 * E.nth;
            }
            const int bm = E.flags >> 4;
            int nf = 0;
            for (int ij = 0; ij < C.nx * C.ny && nf < kMaxFaceNodes; ++ij) {
                const int i = ij / C.ny, j = ij % C.ny;
                bool hit = false;
                if (!bdry(bm, i, j, C.nx, C.ny))
                    for (int F = 0; F < 4; ++F) hit |= ((fm >> F) & 1) && onf(F, i, j, C.nx, C.ny);
                if (hit) {
                    R.push_back(ij);
                    ++nf;
                }
            }
            R[kRecNf] = nf;
            rmax = std::max(rmax, R.size());
        }
        s->rec_stride = (int)((rmax + 31) / 32 * 32);
        if (s->rec_stride > kRecMax) throw RtgError{RTG_ERR_SIZE, "sweep element record too long"};
        std::vector<int32_t> flat((size_t)ne * s->rec_stride, 0);
        for (int idx = 0; idx < ne; ++idx)
            std::copy(recs[idx].begin(), recs[idx].end(), flat.begin() + (size_t)idx * s->rec_stride);
        s->d_rec = sw_alloc<int32_t>(s, flat.size());
        RTG_CUDA(cudaMemcpy(s->d_rec, flat.data(), sizeof(int32_t) * flat.size(), cudaMemcpyHostToDevice));
    }
    return s;
}

// z = P^{-1} r (full-length vectors; inflow-boundary entries of z are zero).
// With trace, element e records in trace[8e .. 8e+7]: claimed, independent
// work done, published (globaltimer ns), its CTA, then SM clock cycles of
// the phases after that: waiting for the upwind lines, forming T, forming the
// couplings, the face columns of B and the stores.
template <typename T>
void apply_sweep(rtg_handle* h, const T* r, T* z, cudaStream_t st, unsigned long long* trace, const int32_t* skip,
                 const int* stop, bool prefilled) {
    Sweep* s = get_sweep(h, st);
    const bool f64 = sizeof(T) == 8;
    using TB = typename BlockStore<T>::type;
    const TB* inv = f64 ? (const TB*)(const void*)s->d_inv64 : (const TB*)(const void*)s->d_inv16;
    OpView<T> v = *reinterpret_cast<const OpView<T>*>(f64 ? (const void*)&h->v64 : (const void*)&h->v32);
    v.skip = skip;
    v.stop = stop;
    if (!prefilled) {
        const int ne = (int)h->host.elems.size();
        sweep_fill_kernel<T><<<std::max(1, std::min(ne, 152 * 8)), 256, 0, st>>>(v, ne, z, s->d_next), count_launch();
    }
    const int pi = f64 ? 1 : 0;
    const int rhs_cap = (std::max(s->max_nloc, 1) + 1) & ~1;   // even: 16-byte aligned region after rhs, zpre
    UpwindMap<T> um;
    um.up = s->d_up;
    using TG = typename MapStore<T>::type;
    um.G = f64 ? (const TG*)(const void*)s->d_G64 : (const TG*)(const void*)s->d_G16;
    auto launch = [&](const Sweep::Shape& sh) {
        um.reg_cap = sh.reg_cap;
        um.stage_cap = (int)(sh.smem / sizeof(T)) - 2 * rhs_cap;
        sweep_persistent_kernel<T><<<sh.grid, sh.threads, sh.smem, st>>>(
            v, s->d_rec, s->rec_stride, (int)h->host.elems.size(), s->d_active, inv, r, z, s->d_next, s->d_status,
            um, rhs_cap, sh.bcap, trace), count_launch();
    };
    if (s->pick[pi] < 0) {
        // the launch shapes: larger per-CTA shared memory (more one-phase
        // elements and staged blocks, fewer CTAs per SM) or smaller (more
        // CTAs per SM and so more element stagings in flight, for meshes whose
        // levels hold many elements; the sweep is throughput bound there)
        int dev = 0, nsm = 0;
        RTG_CUDA(cudaGetDevice(&dev));
        RTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        for (int q = 0; q < kSweepShapes; ++q) {
            Sweep::Shape& sh = s->shape[pi][q];
            const size_t budget = kShapeBudget[q];
            sh.threads = kShapeThreads[q];
            const size_t rhs_bytes = sizeof(T) * (size_t)(2 * rhs_cap + s->max_c);
            const int64_t fit = (int64_t)((budget - std::min(rhs_bytes, budget)) / sizeof(T));
            sh.bcap = (int)std::max<int64_t>(0, std::min<int64_t>(block_units<T, TB>((int)s->max_b), fit));
            sh.reg_cap = (int)std::max<int64_t>(0, (int64_t)(budget / sizeof(T)) - 2 * rhs_cap);
            const int64_t gmax = std::min<int64_t>(f64 ? s->gmax64 : s->gmax32, sh.reg_cap);
            sh.smem = sizeof(T) * (size_t)(2 * rhs_cap + std::max<int64_t>((int64_t)sh.bcap + s->max_c, gmax));
            raise_smem_limit((const void*)sweep_persistent_kernel<T>, sh.smem);
            int per_sm = 0;
            RTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_persistent_kernel<T>, sh.threads,
                                                                   sh.smem));
            sh.grid = std::max(1, std::min<int>((int)h->host.elems.size(), std::max(per_sm, 1) * nsm));
        }
        // time each: rounds over all shapes (so that a drift of the clocks
        // meets every shape alike), the first round a warm-up, best of the
        // other five; a smaller budget must win by 3 %
        cudaEvent_t e0, e1;
        RTG_CUDA(cudaEventCreate(&e0));
        RTG_CUDA(cudaEventCreate(&e1));
        for (int q = 0; q < kSweepShapes; ++q) s->shape_ms[pi][q] = 1e30f;
        for (int rep = 0; rep < 6; ++rep)
            for (int q = 0; q < kSweepShapes; ++q) {
                sweep_fill_kernel<T><<<std::max(1, std::min((int)h->host.elems.size(), 152 * 8)), 256, 0, st>>>(
                    v, (int)h->host.elems.size(), z, s->d_next), count_launch();
                RTG_CUDA(cudaEventRecord(e0, st));
                launch(s->shape[pi][q]);
                RTG_CUDA(cudaEventRecord(e1, st));
                RTG_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                RTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (rep > 0) s->shape_ms[pi][q] = std::min(s->shape_ms[pi][q], ms);
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        int best_q = 0;
        for (int q = 1; q < kSweepShapes; ++q)
            if (s->shape_ms[pi][q] < 0.97f * s->shape_ms[pi][best_q]) best_q = q;
        s->pick[pi] = best_q;
        // the real sweep below starts from a fresh fill
        sweep_fill_kernel<T><<<std::max(1, std::min((int)h->host.elems.size(), 152 * 8)), 256, 0, st>>>(
            v, (int)h->host.elems.size(), z, s->d_next), count_launch();
    }
    launch(s->shape[pi][s->pick[pi]]);
    RTG_CUDA(cudaGetLastError());
}

template <typename T>
void apply_sweep(rtg_handle* h, const T* r, T* z, cudaStream_t st) {
    apply_sweep<T>(h, r, z, st, nullptr);
}

// one-phase elements of a precision, and the map entries and upwind indices
// one sweep in that precision reads
void sweep_maps(rtg_handle* h, int prec, int* onephase, int64_t* map_entries, int64_t* upwind, cudaStream_t st) {
    Sweep* s = get_sweep(h, st);
    const int p = prec == RTG_FP64 ? 1 : 0;
    // the maps the chosen launch shape reads (every element with a map before
    // the first sweep has chosen one)
    const int64_t cap = s->pick[p] >= 0 ? s->shape[p][s->pick[p]].reg_cap : std::numeric_limits<int64_t>::max();
    int n = 0;
    int64_t ent = 0, nup = 0;
    for (const Sweep::MapUse& u : s->onephase[p])
        if (u.region <= cap) {
            ++n;
            ent += u.entries;
            nup += u.nup;
        }
    if (onephase) *onephase = n;
    if (map_entries) *map_entries = ent;
    if (upwind) *upwind = nup;
}

// level of each element in the sweep order (host array of nelem)
void sweep_levels(rtg_handle* h, int32_t* level, cudaStream_t st) {
    Sweep* s = get_sweep(h, st);
    for (int L = 0; L < s->nlev; ++L)
        for (int q = s->lev_start[L]; q < s->lev_start[L + 1]; ++q) level[s->h_lev_elems[q]] = L;
}

// RTG_OK, or RTG_ERR_TIMEOUT if a sweep wait gave up since the last check.
int sweep_status(rtg_handle* h, cudaStream_t st) {
    Sweep* s = h->sweep;
    if (!s) return RTG_OK;
    int status = 0;
    RTG_CUDA(cudaMemcpyAsync(&status, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    RTG_CUDA(cudaStreamSynchronize(st));
    if (status) RTG_CUDA(cudaMemsetAsync(s->d_status, 0, sizeof(int), st));
    return status;
}

template void apply_sweep<double>(rtg_handle*, const double*, double*, cudaStream_t);
template void apply_sweep<float>(rtg_handle*, const float*, float*, cudaStream_t);
template void apply_sweep<double>(rtg_handle*, const double*, double*, cudaStream_t, unsigned long long*,
                                  const int32_t*, const int*, bool);
template void apply_sweep<float>(rtg_handle*, const float*, float*, cudaStream_t, unsigned long long*,
                                 const int32_t*, const int*, bool);

unsigned int* sweep_counter(rtg_handle* h, cudaStream_t st) { return get_sweep(h, st)->d_next; }

int sweep_levels_count(rtg_handle* h, cudaStream_t st) { return get_sweep(h, st)->nlev; }
int sweep_lagged_count(rtg_handle* h, cudaStream_t st) { return get_sweep(h, st)->n_lagged; }
int64_t sweep_inverse_entries(rtg_handle* h, cudaStream_t st) { return get_sweep(h, st)->inv_entries; }

}  // namespace rtg

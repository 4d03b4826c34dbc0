// Learned correction of the sweep preconditioner.
//
// Preconditioner 3 of rtg_solve is M(r) = z + L z with z = P_sweep^{-1} r and
// L a learned operator that is LINEAR in z: the sweep inverts streaming and
// extinction only, so what it leaves is the error that scattering spreads over
// directions and elements, mostly the angle-averaged part in optically thick,
// highly scattering regions.  L acts per row = (element e, spatial node ij):
//
//   m(z) = [m0, m1c, m1s, phi, em, cm, nm, 0]   (8 linear functionals of z)
//     m0, m1c, m1s = sum_a w_a (1, cos th_a, sin th_a) z_a / sum_a w_a  (element e at ij)
//     phi = column angular mean at ij, em = element mean of m0, cm = column
//     mean of phi, nm = mean of cm over the face-neighbour columns
//   o = C(row) m,  C = 3 x 8 coefficients
//   (L z)_(e, ij, a) = o0 + o1 cos th_a + o2 sin th_a   at the unknowns
//
// The coefficients C(row) come from a 16-128-128-24 ReLU network of local
// physics only (optical thickness and albedo at the node and around the
// column, the cell's direction and extent, degrees, boundary faces), times the
// gate g = s / (1 + s), s = sigma h the node's scattering optical thickness:
// where a region neither scatters nor is thick the sweep is already close to
// exact and the correction is switched off whatever the network says.  M is a
// fixed linear operator per problem: the coefficients are computed once when
// the network is set, and each application costs a column pass and an element
// pass over z.  Weights are rounded to BF16 when staged; accumulation is FP32.
//
// Training reduces the loss of a residual -> error pair to per-row statistics
// of the target t = (e - z)/s (s = rms z): G = sum_a b_a b_a^T, q = sum_a b_a
// t_a, c = sum_a t_a^2 with b_a = (1, cos th_a, sin th_a), so that
//   loss = sum_rows o^T G o - 2 q^T o + c,  o = C(row) m(z)/s.
// The gradient kernel recomputes the forward pass per 64-row tile, forms
// dL/dC = (dL/do) m^T, runs the backward pass in shared memory and keeps the
// weight gradients of its tiles in registers; per-CTA partials are summed in a
// fixed order, so training is deterministic.
#include <algorithm>
#include <cmath>

#include <cuda_bf16.h>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kIn = RTG_NN_IN, kHid = RTG_NN_HIDDEN, kOut = RTG_NN_OUT, kMom = RTG_NN_MOM;
constexpr int kSt = RTG_NN_STATS;
constexpr int kTile = 64;          // rows per tile
constexpr int kLd = kTile + 4;     // row stride of the transposed activation tiles
constexpr int kLdo = kOut + 1;     // row stride of dL/dC in shared memory (bank spread)
constexpr int kMlpThreads = 256;
constexpr int kGradCtas = 2 * 152;
constexpr int oW1 = 0, ob1 = oW1 + kIn * kHid, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kHid * kOut, kNP = ob3 + kOut;
static_assert(kNP == RTG_NN_NPARAM, "parameter layout");
static_assert(kOut == 3 * kMom, "three output moments");
static_assert(kOut % 4 == 0, "output rows are float4-aligned");
constexpr float kTwoPi = 6.283185307179586f;

// shared-memory layout of the MLP kernels (floats); the parameter layout is
// the shared-memory layout of the first kNP floats; float4 regions start on
// multiples of 4 floats
constexpr int sF = (kNP + 3) / 4 * 4, sH1 = sF + kIn * kLd, sH2 = sH1 + kHid * kLd, sO = sH2 + kHid * kLd,
              kSmemFloats = sO + kTile * kOut;
static_assert(sF % 4 == 0 && sH1 % 4 == 0 && sH2 % 4 == 0 && sO % 4 == 0, "alignment");
static_assert(oW2 % 4 == 0 && oW1 % 4 == 0, "weight rows are float4-aligned");
constexpr size_t kMlpSmem = sizeof(float) * kSmemFloats;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ bool bdry_node_n(int bm, int i, int j, int nx, int ny) {
    return ((bm & 1) && i == nx - 1) || ((bm & 2) && j == ny - 1) || ((bm & 4) && i == 0) ||
           ((bm & 8) && j == 0);
}

__device__ void stage_params(const float* __restrict__ P, float* sm) {
    for (int t = threadIdx.x; t < kNP; t += blockDim.x) {
        const bool weight = t < ob1 || (t >= oW2 && t < ob2) || (t >= oW3 && t < ob3);
        const float val = P[t];
        sm[t] = weight ? bf16r(val) : val;
    }
}

// outT[c][r] = relu(sum_k inT[k][r] W[k][c] + b[c]) for the 64-row tile;
// thread: rows 4tr..4tr+3, columns 8tc..8tc+7
template <int K>
__device__ __forceinline__ void layer_relu(const float* __restrict__ inT, const float* __restrict__ W,
                                           const float* __restrict__ b, float* __restrict__ outT) {
    const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
        const float4 a = *reinterpret_cast<const float4*>(inT + k * kLd + 4 * tr);
        const float4 w0 = *reinterpret_cast<const float4*>(W + k * kHid + 8 * tc);
        const float4 w1 = *reinterpret_cast<const float4*>(W + k * kHid + 8 * tc + 4);
        const float av[4] = {a.x, a.y, a.z, a.w};
        const float wv[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], wv[j], acc[i][j]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float bj = b[8 * tc + j];
        float4 o;
        o.x = fmaxf(acc[0][j] + bj, 0.f);
        o.y = fmaxf(acc[1][j] + bj, 0.f);
        o.z = fmaxf(acc[2][j] + bj, 0.f);
        o.w = fmaxf(acc[3][j] + bj, 0.f);
        *reinterpret_cast<float4*>(outT + (8 * tc + j) * kLd + 4 * tr) = o;
    }
}

// gate of a row from its features: s = c (e^f0 - 1) = sigma h, g = s / (1 + s)
__device__ __forceinline__ float row_gate(float f0, float f1) {
    const float sv = fmaxf(f1 * expm1f(f0), 0.f);
    return sv / (1.f + sv);
}

// Forward pass of one tile: features into Ft, then h1T, h2T and the gated
// outputs in sO[r][kOut] (thread: row t/4, outputs t%4 + 4u).
__device__ __forceinline__ void forward_tile(const float* __restrict__ F, int64_t r0, int nr, float* sm) {
    float* Ft = sm + sF;
    for (int t = threadIdx.x; t < kTile * kIn; t += blockDim.x) {
        const int r = t / kIn, k = t % kIn;
        Ft[k * kLd + r] = r < nr ? F[(r0 + r) * kIn + k] : 0.f;
    }
    __syncthreads();
    layer_relu<kIn>(Ft, sm + oW1, sm + ob1, sm + sH1);
    __syncthreads();
    layer_relu<kHid>(sm + sH1, sm + oW2, sm + ob2, sm + sH2);
    __syncthreads();
    const int r = threadIdx.x >> 2, c0 = threadIdx.x & 3;
    const float* h2T = sm + sH2;
    const float* W3 = sm + oW3;
    float acc[kOut / 4];
#pragma unroll
    for (int u = 0; u < kOut / 4; ++u) acc[u] = sm[ob3 + c0 + 4 * u];
#pragma unroll 4
    for (int k = 0; k < kHid; ++k) {
        const float hv = h2T[k * kLd + r];
#pragma unroll
        for (int u = 0; u < kOut / 4; ++u) acc[u] = fmaf(hv, W3[k * kOut + c0 + 4 * u], acc[u]);
    }
    const float g = row_gate(Ft[r], Ft[kLd + r]);
#pragma unroll
    for (int u = 0; u < kOut / 4; ++u) sm[sO + r * kOut + c0 + 4 * u] = g * acc[u];
    __syncthreads();
}

__global__ void __launch_bounds__(kMlpThreads, 1)
nn_forward_kernel(const float* __restrict__ P, const float* __restrict__ F, int64_t rows, float* __restrict__ O) {
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    stage_params(P, sm);
    __syncthreads();
    const int64_t ntiles = (rows + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t r0 = tile * kTile;
        const int nr = (int)(rows - r0 < kTile ? rows - r0 : kTile);
        forward_tile(F, r0, nr, sm);
        for (int t = threadIdx.x; t < nr * kOut; t += blockDim.x) O[r0 * kOut + t] = sm[sO + t];
        __syncthreads();
    }
}

// Loss and gradient over all rows.  work[b][kNP] gets CTA b's gradient,
// lossw[b] its loss.
__global__ void __launch_bounds__(kMlpThreads, 1)
nn_grad_kernel(const float* __restrict__ P, const float* __restrict__ F, const float* __restrict__ Mo,
               const float* __restrict__ S, int64_t rows, float* __restrict__ work, double* __restrict__ lossw) {
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    __shared__ float dO[kTile * kLdo];
    __shared__ double red[kMlpThreads / 32];
    stage_params(P, sm);
    __syncthreads();
    const int t = threadIdx.x;
    constexpr int kW3PerThread = kHid * kOut / kMlpThreads;
    float gW2[8][8], gW1[8], gW3[kW3PerThread], gb1 = 0.f, gb2 = 0.f, gb3 = 0.f;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        gW1[p] = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) gW2[p][q] = 0.f;
    }
#pragma unroll
    for (int u = 0; u < kW3PerThread; ++u) gW3[u] = 0.f;
    double loss = 0.;
    float* Ft = sm + sF;
    float* h1T = sm + sH1;
    float* h2T = sm + sH2;
    const float* W2 = sm + oW2;
    const float* W3 = sm + oW3;
    const int64_t ntiles = (rows + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t r0 = tile * kTile;
        const int nr = (int)(rows - r0 < kTile ? rows - r0 : kTile);
        forward_tile(F, r0, nr, sm);
        // o = C m, loss, dL/dC = (dL/do) m^T
        if (t < kTile) {
            float m[kMom], d[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int l = 0; l < kMom; ++l) m[l] = 0.f;
            if (t < nr) {
                const float* s = S + (r0 + t) * kSt;
                const float* mg = Mo + (r0 + t) * kMom;
#pragma unroll
                for (int l = 0; l < kMom; ++l) m[l] = mg[l];
                float o[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float a = 0.f;
#pragma unroll
                    for (int l = 0; l < kMom; ++l) a = fmaf(sm[sO + t * kOut + kMom * k + l], m[l], a);
                    o[k] = a;
                }
                const float g0 = s[0] * o[0] + s[1] * o[1] + s[2] * o[2];
                const float g1 = s[1] * o[0] + s[3] * o[1] + s[4] * o[2];
                const float g2 = s[2] * o[0] + s[4] * o[1] + s[5] * o[2];
                loss += (double)(o[0] * g0 + o[1] * g1 + o[2] * g2) -
                        2. * (double)(s[6] * o[0] + s[7] * o[1] + s[8] * o[2]) + (double)s[9];
                d[0] = 2.f * (g0 - s[6]);
                d[1] = 2.f * (g1 - s[7]);
                d[2] = 2.f * (g2 - s[8]);
            }
            // dL/d(pre-gate outputs) = g dL/dC
            const float g = row_gate(Ft[t], Ft[kLd + t]);
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int l = 0; l < kMom; ++l) dO[t * kLdo + kMom * k + l] = g * d[k] * m[l];
        }
        __syncthreads();
        // dW3, db3
#pragma unroll
        for (int u = 0; u < kW3PerThread; ++u) {
            const int idx = t + kMlpThreads * u, k = idx / kOut, c = idx % kOut;
            float a = 0.f;
            for (int r = 0; r < kTile; ++r) a = fmaf(h2T[k * kLd + r], dO[r * kLdo + c], a);
            gW3[u] += a;
        }
        if (t < kOut)
            for (int r = 0; r < kTile; ++r) gb3 += dO[r * kLdo + t];
        __syncthreads();
        // dh2 = (dO W3^T) * [h2 > 0], in place
        {
            const int tr = t & 15, tc = t >> 4;
#pragma unroll 2
            for (int j = 0; j < 8; ++j) {
                const int k = 8 * tc + j;
                float4 hv = *reinterpret_cast<float4*>(h2T + k * kLd + 4 * tr);
                float* hp = &hv.x;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 4 * tr + i;
                    float dsum = 0.f;
#pragma unroll
                    for (int c = 0; c < kOut; ++c) dsum = fmaf(dO[r * kLdo + c], W3[k * kOut + c], dsum);
                    hp[i] = hp[i] > 0.f ? dsum : 0.f;
                }
                *reinterpret_cast<float4*>(h2T + k * kLd + 4 * tr) = hv;
            }
        }
        __syncthreads();
        if (t < kHid)
            for (int r = 0; r < kTile; ++r) gb2 += h2T[t * kLd + r];
        // dW2[k][c] += sum_r h1[r][k] dh2[r][c]; k = tk + 16p, c = 8tc + q
        {
            const int tk = t & 15, tc = t >> 4;
            for (int r = 0; r < kTile; r += 4) {
                float4 a[8], b[8];
#pragma unroll
                for (int p = 0; p < 8; ++p) a[p] = *reinterpret_cast<const float4*>(h1T + (tk + 16 * p) * kLd + r);
#pragma unroll
                for (int q = 0; q < 8; ++q) b[q] = *reinterpret_cast<const float4*>(h2T + (8 * tc + q) * kLd + r);
#pragma unroll
                for (int p = 0; p < 8; ++p)
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        gW2[p][q] = fmaf(a[p].x, b[q].x,
                                         fmaf(a[p].y, b[q].y, fmaf(a[p].z, b[q].z, fmaf(a[p].w, b[q].w, gW2[p][q]))));
            }
        }
        __syncthreads();
        // dh1 = (dh2 W2^T) * [h1 > 0], in place; rows 4tr.., k = tk + 16p
        {
            const int tr = t & 15, tk = t >> 4;
            float acc[8][4];
#pragma unroll
            for (int p = 0; p < 8; ++p)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[p][i] = 0.f;
#pragma unroll 2
            for (int c = 0; c < kHid; ++c) {
                const float4 d = *reinterpret_cast<const float4*>(h2T + c * kLd + 4 * tr);
#pragma unroll
                for (int p = 0; p < 8; ++p) {
                    const float w = W2[(tk + 16 * p) * kHid + c];
                    acc[p][0] = fmaf(d.x, w, acc[p][0]);
                    acc[p][1] = fmaf(d.y, w, acc[p][1]);
                    acc[p][2] = fmaf(d.z, w, acc[p][2]);
                    acc[p][3] = fmaf(d.w, w, acc[p][3]);
                }
            }
#pragma unroll
            for (int p = 0; p < 8; ++p) {
                float4 hv = *reinterpret_cast<float4*>(h1T + (tk + 16 * p) * kLd + 4 * tr);
                hv.x = hv.x > 0.f ? acc[p][0] : 0.f;
                hv.y = hv.y > 0.f ? acc[p][1] : 0.f;
                hv.z = hv.z > 0.f ? acc[p][2] : 0.f;
                hv.w = hv.w > 0.f ? acc[p][3] : 0.f;
                *reinterpret_cast<float4*>(h1T + (tk + 16 * p) * kLd + 4 * tr) = hv;
            }
        }
        __syncthreads();
        if (t < kHid)
            for (int r = 0; r < kTile; ++r) gb1 += h1T[t * kLd + r];
        // dW1[k][c] += sum_r F[r][k] dh1[r][c]; k = t & 15, c = 8 (t >> 4) + q
        {
            const int k = t & 15, c0 = 8 * (t >> 4);
            for (int r = 0; r < kTile; r += 4) {
                const float4 a = *reinterpret_cast<const float4*>(Ft + k * kLd + r);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 b = *reinterpret_cast<const float4*>(h1T + (c0 + q) * kLd + r);
                    gW1[q] = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, gW1[q]))));
                }
            }
        }
        __syncthreads();
    }
    // per-CTA partials
    float* g = work + (int64_t)blockIdx.x * kNP;
    {
        const int tk = t & 15, tc = t >> 4;
#pragma unroll
        for (int p = 0; p < 8; ++p)
#pragma unroll
            for (int q = 0; q < 8; ++q) g[oW2 + (tk + 16 * p) * kHid + 8 * tc + q] = gW2[p][q];
        const int k = t & 15, c0 = 8 * (t >> 4);
#pragma unroll
        for (int q = 0; q < 8; ++q) g[oW1 + k * kHid + c0 + q] = gW1[q];
#pragma unroll
        for (int u = 0; u < kW3PerThread; ++u) g[oW3 + t + kMlpThreads * u] = gW3[u];
        if (t < kHid) {
            g[ob1 + t] = gb1;
            g[ob2 + t] = gb2;
        }
        if (t < kOut) g[ob3 + t] = gb3;
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
    if ((t & 31) == 0) red[t >> 5] = loss;
    __syncthreads();
    if (t == 0) {
        double s = 0.;
        for (int w = 0; w < kMlpThreads / 32; ++w) s += red[w];
        lossw[blockIdx.x] = s;
    }
}

__global__ void nn_reduce_grad_kernel(const float* __restrict__ work, int nb, const double* __restrict__ lossw,
                                      float* __restrict__ grad, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < kNP) {
        float s = 0.f;
        for (int b = 0; b < nb; ++b) s += work[(int64_t)b * kNP + p];
        grad[p] = s;
    }
    if (p == 0 && loss) {
        double s = 0.;
        for (int b = 0; b < nb; ++b) s += lossw[b];
        *loss = s;
    }
}

__global__ void nn_adam_kernel(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                               float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float wd,
                               float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * P[i]);
}

// ------------------------------------------------------------ physics features
// Per column: the weighted means over its nodes of tau = log1p(kappa h) and of
// the albedo c = sigma / kappa (one warp per column).
template <typename T>
__global__ void nn_colphys_kernel(OpView<T> v, float* __restrict__ ctau, float* __restrict__ calb) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int ci = blockIdx.x * wpb + (threadIdx.x >> 5); ci < v.ncols; ci += gridDim.x * wpb) {
        const ColDev C = v.cols[ci];
        const T* wx = v.lglw + C.nx * kMaxNodes;
        const T* wy = v.lglw + C.ny * kMaxNodes;
        const float h = (float)fmin(C.dx, C.dy);
        float st = 0.f, sc = 0.f;
        for (int ij = lane; ij < C.nx * C.ny; ij += 32) {
            const int i = ij / C.ny, j = ij % C.ny;
            const float ww = (float)(wx[i] * wy[j]);
            const float kap = (float)v.kw[C.node_off + ij] / ww, sig = (float)v.sw[C.node_off + ij] / ww;
            st = fmaf(0.25f * ww, log1pf(fmaxf(kap, 0.f) * h), st);
            sc = fmaf(0.25f * ww, kap > 0.f ? sig / kap : 0.f, sc);
        }
        for (int o = 16; o > 0; o >>= 1) {
            st += __shfl_down_sync(0xffffffffu, st, o);
            sc += __shfl_down_sync(0xffffffffu, sc, o);
        }
        if (lane == 0) {
            ctau[ci] = st;
            calb[ci] = sc;
        }
    }
}

__device__ __forceinline__ float nbr_mean(const int32_t* __restrict__ nbr8, int ci, const float* __restrict__ a) {
    float s = 0.f;
    int cnt = 0;
    for (int q = 0; q < 8; ++q) {
        const int nb = nbr8[8 * ci + q];
        if (nb >= 0) {
            s += a[nb];
            ++cnt;
        }
    }
    return cnt ? s / (float)cnt : 0.f;
}

// mean of a over the neighbours across face F, or a[ci] without one
__device__ __forceinline__ float face_mean(const int32_t* __restrict__ raw, int ci, int F, const float* __restrict__ a) {
    const int n0 = raw[8 * ci + 2 * F], n1 = raw[8 * ci + 2 * F + 1];
    if (n0 >= 0 && n1 >= 0) return 0.5f * (a[n0] + a[n1]);
    if (n0 >= 0) return a[n0];
    if (n1 >= 0) return a[n1];
    return a[ci];
}

// One warp per element: the 16 physics features of each of its rows.
template <typename T>
__global__ void nn_physfeat_kernel(OpView<T> v, const float* __restrict__ ctau, const float* __restrict__ calb,
                                   const int32_t* __restrict__ nbr8, const int32_t* __restrict__ raw,
                                   const int32_t* __restrict__ nfree, const int64_t* __restrict__ row_off,
                                   float* __restrict__ feat) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < v.nelem; e += gridDim.x * wpb) {
        const ElemDev E = v.elems[e];
        const int ci = E.col;
        const ColDev C = v.cols[ci];
        const T* A = v.ang + E.ang;
        const int nth = E.nth;
        float sw = 0.f, sc = 0.f, ss = 0.f;
        for (int a = 0; a < nth; ++a) {
            const float w = (float)A[a];
            sw += w;
            sc = fmaf(w, (float)A[3 * nth + a], sc);
            ss = fmaf(w, (float)A[4 * nth + a], ss);
        }
        const float gx = face_mean(raw, ci, 0, ctau) - face_mean(raw, ci, 2, ctau);
        const float gy = face_mean(raw, ci, 1, ctau) - face_mean(raw, ci, 3, ctau);
        const float4 f2 = make_float4((float)E.dth / kTwoPi, (float)(C.nx - 1) * 0.125f, (float)(nth - 1) * 0.125f,
                                      (float)nfree[ci] * 0.25f);
        const float4 f3a = make_float4(ctau[ci], nbr_mean(nbr8, ci, ctau), calb[ci], nbr_mean(nbr8, ci, calb));
        const float gn = sqrtf(gx * gx + gy * gy);
        const float h = (float)fmin(C.dx, C.dy);
        const T* wx = v.lglw + C.nx * kMaxNodes;
        const T* wy = v.lglw + C.ny * kMaxNodes;
        for (int ij = lane; ij < C.nx * C.ny; ij += 32) {
            const int i = ij / C.ny, j = ij % C.ny;
            const int node = C.node_off + ij;
            const float ww = (float)(wx[i] * wy[j]);
            const float kap = fmaxf((float)v.kw[node] / ww, 0.f), sig = (float)v.sw[node] / ww;
            const float c = kap > 0.f ? sig / kap : 0.f;
            const float px = C.nx > 1 ? 2.f * (float)i / (float)(C.nx - 1) - 1.f : 0.f;
            const float py = C.ny > 1 ? 2.f * (float)j / (float)(C.ny - 1) - 1.f : 0.f;
            float4* f = reinterpret_cast<float4*>(feat + (row_off[e] + ij) * kIn);
            f[0] = make_float4(log1pf(kap * h), c, -logf(fmaxf(1.f - c, 0.f) + 1e-3f),
                               log1pf(fmaxf(kap - sig, 0.f) * h));
            f[1] = make_float4(sc / sw, ss / sw, f2.x, f2.y);
            f[2] = make_float4(f2.z, f2.w, f3a.x, f3a.y);
            f[3] = make_float4(f3a.z, f3a.w, px * gx + py * gy, gn);
        }
    }
}

// ------------------------------------------------------------- z moments
// Per column: angular mean phi at each node, the element means em, the column
// mean cm of phi and, when colsq is given, sum z^2 over the column.  One thread
// per (cell, node) forms the node's angular sums; the sums over cells (phi) and
// over nodes (em, cm, colsq) run in a fixed order, so the result does not
// depend on the schedule.  Shared memory: s0w[ncell][nij] (w-weighted sums),
// swt[ncell] (angular weight sums), and, with colsq, sqs[ncell][nij].
template <typename T>
__global__ void nn_colstats_kernel(OpView<T> v, const T* __restrict__ z, float* __restrict__ phi,
                                   float* __restrict__ em, float* __restrict__ cm, double* __restrict__ colsq) {
    extern __shared__ float sm[];
    if (v.stop && *v.stop) return;
    const ColDev C = v.cols[blockIdx.x];
    const int nij = C.nx * C.ny, ncell = C.elem_end - C.elem_begin;
    float* s0w = sm;                           // [ncell][nij]
    float* swt = s0w + ncell * nij;            // [ncell]
    float* phs = swt + ncell;                  // [nij]
    float* sqs = phs + nij;                    // [ncell][nij] (colsq only)
    const T* wx = v.lglw + C.nx * kMaxNodes;
    const T* wy = v.lglw + C.ny * kMaxNodes;
    for (int t = threadIdx.x; t < ncell * nij; t += blockDim.x) {
        const int k = t / nij, ij = t % nij;
        const ElemDev E = v.elems[C.elem_begin + k];
        const T* A = v.ang + E.ang;
        const T* ze = z + E.dof_off + (int64_t)ij * E.nth;
        float s0 = 0.f, sw = 0.f, sq = 0.f;
        for (int a = 0; a < E.nth; ++a) {
            const float zv = (float)ze[a];
            const float w = (float)A[a];
            s0 = fmaf(w, zv, s0);
            sw += w;
            sq = fmaf(zv, zv, sq);
        }
        s0w[t] = s0;
        if (ij == 0) swt[k] = sw;
        if (colsq) sqs[t] = sq;
    }
    __syncthreads();
    // phi per node: cells in order
    for (int ij = threadIdx.x; ij < nij; ij += blockDim.x) {
        float ph = 0.f;
        for (int k = 0; k < ncell; ++k) ph = fmaf((float)v.elems[C.elem_begin + k].dth * 0.5f, s0w[k * nij + ij], ph);
        ph /= kTwoPi;
        phi[C.node_off + ij] = ph;
        phs[ij] = ph;
    }
    // element means: one warp per cell, lanes over nodes, fixed shuffle tree
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = wid; k < ncell; k += nw) {
        float acc = 0.f;
        for (int ij = lane; ij < nij; ij += 32)
            acc = fmaf((float)(wx[ij / C.ny] * wy[ij % C.ny]) * 0.25f, s0w[k * nij + ij], acc);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) em[C.elem_begin + k] = acc / swt[k];
    }
    __syncthreads();
    if (wid == 0) {
        float c = 0.f;
        for (int ij = lane; ij < nij; ij += 32) c = fmaf((float)(wx[ij / C.ny] * wy[ij % C.ny]) * 0.25f, phs[ij], c);
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
        if (lane == 0) cm[blockIdx.x] = c;
    }
    if (colsq && threadIdx.x < 32) {
        double sq = 0.;
        for (int t = threadIdx.x; t < ncell * nij; t += 32) sq += (double)sqs[t];
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
        if (threadIdx.x == 0) colsq[blockIdx.x] = sq;
    }
}

__global__ void nn_scale_kernel(const double* __restrict__ colsq, int ncols, double n, float* __restrict__ scale) {
    __shared__ double red[32];
    double s = 0.;
    for (int i = threadIdx.x; i < ncols; i += blockDim.x) s += colsq[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += red[w];
        const double r = sqrt(t / n);
        scale[0] = r == 0. ? 1.f : (float)r;
    }
}

// the eight moments of row (e, ij) of z; em, cm, nm are per element/column
template <typename T>
__device__ __forceinline__ void row_moments(const T* __restrict__ ze, const T* __restrict__ A, int nth, float isw,
                                            float ph, float emv, float cmv, float nmv, float* m) {
    float m0 = 0.f, m1 = 0.f, m2 = 0.f;
    for (int a = 0; a < nth; ++a) {
        const float wz = (float)A[a] * (float)ze[a];
        m0 += wz;
        m1 = fmaf(wz, (float)A[3 * nth + a], m1);
        m2 = fmaf(wz, (float)A[4 * nth + a], m2);
    }
    m[0] = m0 * isw;
    m[1] = m1 * isw;
    m[2] = m2 * isw;
    m[3] = ph;
    m[4] = emv;
    m[5] = cmv;
    m[6] = nmv;
    m[7] = 0.f;
}

// One warp per element: mom[row][8] = m(z) / s.
template <typename T>
__global__ void nn_moments_kernel(OpView<T> v, const T* __restrict__ z, const float* __restrict__ phi,
                                  const float* __restrict__ em, const float* __restrict__ cm,
                                  const int32_t* __restrict__ nbr8, const int64_t* __restrict__ row_off,
                                  const float* __restrict__ scale, float* __restrict__ mom) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const float is = 1.f / scale[0];
    for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < v.nelem; e += gridDim.x * wpb) {
        const ElemDev E = v.elems[e];
        const ColDev C = v.cols[E.col];
        const T* A = v.ang + E.ang;
        float sw = 0.f;
        for (int a = 0; a < E.nth; ++a) sw += (float)A[a];
        const float nmv = nbr_mean(nbr8, E.col, cm);
        for (int ij = lane; ij < C.nx * C.ny; ij += 32) {
            float m[kMom];
            row_moments(z + E.dof_off + (int64_t)ij * E.nth, A, E.nth, 1.f / sw, phi[C.node_off + ij], em[e],
                        cm[E.col], nmv, m);
            float4* o = reinterpret_cast<float4*>(mom + (row_off[e] + ij) * kMom);
            o[0] = make_float4(m[0] * is, m[1] * is, m[2] * is, m[3] * is);
            o[1] = make_float4(m[4] * is, m[5] * is, m[6] * is, 0.f);
        }
    }
}

// One warp per element: z += o0 + o1 cos th + o2 sin th at the unknowns,
// o = C(row) m(z).  Each row reads only its own entries of z before writing
// them; the aggregates come from nn_colstats_kernel.
template <typename T>
__global__ void nn_correct_kernel(OpView<T> v, const float* __restrict__ coef, const float* __restrict__ phi,
                                  const float* __restrict__ em, const float* __restrict__ cm,
                                  const int32_t* __restrict__ nbr8, const int64_t* __restrict__ row_off,
                                  T* __restrict__ z) {
    if (v.stop && *v.stop) return;
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < v.nelem; e += gridDim.x * wpb) {
        const ElemDev E = v.elems[e];
        const ColDev C = v.cols[E.col];
        const T* A = v.ang + E.ang;
        const int nth = E.nth, bm = E.flags >> 4;
        float sw = 0.f;
        for (int a = 0; a < nth; ++a) sw += (float)A[a];
        const float nmv = nbr_mean(nbr8, E.col, cm);
        for (int ij = lane; ij < C.nx * C.ny; ij += 32) {
            const int i = ij / C.ny, j = ij % C.ny;
            if (bdry_node_n(bm, i, j, C.nx, C.ny)) continue;
            T* ze = z + E.dof_off + (int64_t)ij * nth;
            float m[kMom];
            row_moments(ze, A, nth, 1.f / sw, phi[C.node_off + ij], em[e], cm[E.col], nmv, m);
            const float4* cr = reinterpret_cast<const float4*>(coef + (row_off[e] + ij) * kOut);
            float o[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 c0 = cr[2 * k], c1 = cr[2 * k + 1];
                o[k] = c0.x * m[0] + c0.y * m[1] + c0.z * m[2] + c0.w * m[3] + c1.x * m[4] + c1.y * m[5] +
                       c1.z * m[6] + c1.w * m[7];
            }
            for (int a = 0; a < nth; ++a)
                ze[a] += (T)(o[0] + o[1] * (float)A[3 * nth + a] + o[2] * (float)A[4 * nth + a]);
        }
    }
}

// Training statistics of the target t = (e - z)/s per row (times weight).
template <typename T>
__global__ void nn_stats_kernel(OpView<T> v, const T* __restrict__ z, const T* __restrict__ err,
                                const int64_t* __restrict__ row_off, const float* __restrict__ scale, float weight,
                                float* __restrict__ S) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const double is = 1. / (double)scale[0];
    for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < v.nelem; e += gridDim.x * wpb) {
        const ElemDev E = v.elems[e];
        const ColDev C = v.cols[E.col];
        const T* A = v.ang + E.ang;
        const int nth = E.nth, bm = E.flags >> 4, nij = C.nx * C.ny;
        for (int ij = lane; ij < nij; ij += 32) {
            const int i = ij / C.ny, j = ij % C.ny;
            float g[12];
#pragma unroll
            for (int q = 0; q < 12; ++q) g[q] = 0.f;
            if (!bdry_node_n(bm, i, j, C.nx, C.ny)) {
                const int64_t b0 = E.dof_off + (int64_t)ij * nth;
                for (int a = 0; a < nth; ++a) {
                    const float tv = (float)(((double)err[b0 + a] - (double)z[b0 + a]) * is);
                    const float c = (float)A[3 * nth + a], sn = (float)A[4 * nth + a];
                    g[0] += 1.f;
                    g[1] += c;
                    g[2] += sn;
                    g[3] = fmaf(c, c, g[3]);
                    g[4] = fmaf(c, sn, g[4]);
                    g[5] = fmaf(sn, sn, g[5]);
                    g[6] += tv;
                    g[7] = fmaf(c, tv, g[7]);
                    g[8] = fmaf(sn, tv, g[8]);
                    g[9] = fmaf(tv, tv, g[9]);
                }
#pragma unroll
                for (int q = 0; q < 10; ++q) g[q] *= weight;
            }
            float4* o = reinterpret_cast<float4*>(S + (row_off[e] + ij) * kSt);
            o[0] = make_float4(g[0], g[1], g[2], g[3]);
            o[1] = make_float4(g[4], g[5], g[6], g[7]);
            o[2] = make_float4(g[8], g[9], g[10], g[11]);
        }
    }
}

inline int elem_grid(int n) { return std::max(1, std::min((n + 7) / 8, 152 * 16)); }

template <typename T>
const OpView<T>& nview(const rtg_handle* h);
template <>
const OpView<double>& nview<double>(const rtg_handle* h) { return h->v64; }
template <>
const OpView<float>& nview<float>(const rtg_handle* h) { return h->v32; }

}  // namespace

struct NNWs {
    int64_t rows = 0;
    int64_t* row_off = nullptr;   // [nelem + 1]
    int32_t* nbr8 = nullptr;      // [ncols][8] distinct neighbours
    int32_t* raw = nullptr;       // [ncols][4][2] neighbours per face
    int32_t* nfree = nullptr;     // [ncols]
    float* ctau = nullptr;        // [ncols]
    float* calb = nullptr;        // [ncols]
    float* phi = nullptr;         // [nnodes]
    float* cm = nullptr;          // [ncols]
    float* em = nullptr;          // [nelem]
    double* colsq = nullptr;      // [ncols]
    float* feat = nullptr;        // [rows][16] physics features
    float* coef = nullptr;        // [rows][24] coefficients of the handle's network
    bool has_params = false;
    std::vector<void*> allocs;
};

static void mlp_attributes() {
    raise_smem_limit((const void*)nn_forward_kernel, kMlpSmem);
    raise_smem_limit((const void*)nn_grad_kernel, kMlpSmem);
}

static void* nn_alloc(NNWs* w, size_t bytes) {
    void* p = nullptr;
    RTG_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
    w->allocs.push_back(p);
    return p;
}

template <typename T>
static T* nn_upload(NNWs* w, const std::vector<T>& v) {
    T* p = (T*)nn_alloc(w, sizeof(T) * v.size());
    if (!v.empty()) RTG_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return p;
}

NNWs* get_nn(rtg_handle* h) {
    if (h->nn) return h->nn;
    const HostTables& t = h->host;
    NNWs* w = new NNWs();
    h->nn = w;
    try {
        std::vector<int64_t> ro(t.elems.size() + 1, 0);
        for (size_t e = 0; e < t.elems.size(); ++e) {
            const ColDev& C = t.cols[t.elems[e].col];
            ro[e + 1] = ro[e] + (int64_t)C.nx * C.ny;
        }
        w->rows = ro.back();
        const size_t nc = t.cols.size();
        w->row_off = nn_upload(w, ro);
        w->nbr8 = nn_upload(w, t.col_nbr8);
        w->raw = nn_upload(w, t.col_nbr_raw);
        w->nfree = nn_upload(w, t.col_free);
        w->ctau = (float*)nn_alloc(w, sizeof(float) * nc);
        w->calb = (float*)nn_alloc(w, sizeof(float) * nc);
        w->phi = (float*)nn_alloc(w, sizeof(float) * (size_t)t.nnodes);
        w->cm = (float*)nn_alloc(w, sizeof(float) * nc);
        w->em = (float*)nn_alloc(w, sizeof(float) * t.elems.size());
        w->colsq = (double*)nn_alloc(w, sizeof(double) * nc);
        w->feat = (float*)nn_alloc(w, sizeof(float) * kIn * (size_t)w->rows);
        w->coef = (float*)nn_alloc(w, sizeof(float) * kOut * (size_t)w->rows);
        mlp_attributes();
    } catch (...) {
        free_nn(h);
        throw;
    }
    return w;
}

void free_nn(rtg_handle* h) {
    if (!h->nn) return;
    for (void* p : h->nn->allocs) cudaFree(p);
    delete h->nn;
    h->nn = nullptr;
}

int64_t nn_rows(rtg_handle* h) { return get_nn(h)->rows; }

void nn_features(rtg_handle* h, float* feat, cudaStream_t s) {
    NNWs* w = get_nn(h);
    const OpView<float>& v = h->v32;
    nn_colphys_kernel<float><<<elem_grid(v.ncols), 256, 0, s>>>(v, w->ctau, w->calb), count_launch();
    nn_physfeat_kernel<float><<<elem_grid(v.nelem), 256, 0, s>>>(v, w->ctau, w->calb, w->nbr8, w->raw, w->nfree,
                                                                w->row_off, feat ? feat : w->feat), count_launch();
    RTG_CUDA(cudaGetLastError());
}

void nn_forward(const float* params, const float* feat, int64_t rows, float* coef, cudaStream_t s) {
    if (rows <= 0) return;
    mlp_attributes();
    const int64_t ntiles = (rows + kTile - 1) / kTile;
    const int grid = (int)std::min<int64_t>(ntiles, 152);
    nn_forward_kernel<<<grid, kMlpThreads, kMlpSmem, s>>>(params, feat, rows, coef), count_launch();
    RTG_CUDA(cudaGetLastError());
}

// The coefficients of the handle's problem: physics features, then the network.
void nn_set_params(rtg_handle* h, const float* params, cudaStream_t s) {
    NNWs* w = get_nn(h);
    float* P = nullptr;
    RTG_CUDA(cudaMalloc(&P, sizeof(float) * kNP));
    try {
        RTG_CUDA(cudaMemcpyAsync(P, params, sizeof(float) * kNP, cudaMemcpyDefault, s));
        nn_features(h, w->feat, s);
        nn_forward(P, w->feat, w->rows, w->coef, s);
        RTG_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        cudaFree(P);
        throw;
    }
    RTG_CUDA(cudaFree(P));
    w->has_params = true;
    h->nn_trial[0] = h->nn_trial[1] = 0;   // a new network gets a new trial
}

bool nn_has_params(rtg_handle* h) { return h->nn && h->nn->has_params; }

template <typename T>
static void colstats(rtg_handle* h, NNWs* w, const T* z, bool with_sq, cudaStream_t s, const int* stop = nullptr) {
    OpView<T> v = nview<T>(h);
    v.stop = stop;
    int max_nij = 1;
    for (const ColDev& C : h->host.cols) max_nij = std::max(max_nij, C.nx * C.ny);
    const size_t cells = (size_t)std::max(1, h->host.max_cells_col);
    const size_t smem = sizeof(float) * (cells * max_nij * (with_sq ? 2 : 1) + cells + max_nij);
    raise_smem_limit((const void*)nn_colstats_kernel<T>, smem);
    nn_colstats_kernel<T><<<v.ncols, 128, smem, s>>>(v, z, w->phi, w->em, w->cm, with_sq ? w->colsq : nullptr),
        count_launch();
}

template <typename T>
void nn_moments(rtg_handle* h, const T* z, float* mom, float* scale, cudaStream_t s) {
    NNWs* w = get_nn(h);
    const OpView<T>& v = nview<T>(h);
    colstats<T>(h, w, z, true, s);
    nn_scale_kernel<<<1, 1024, 0, s>>>(w->colsq, v.ncols, (double)h->host.ndof, scale), count_launch();
    nn_moments_kernel<T><<<elem_grid(v.nelem), 256, 0, s>>>(v, z, w->phi, w->em, w->cm, w->nbr8, w->row_off, scale,
                                                           mom), count_launch();
    RTG_CUDA(cudaGetLastError());
}

template <typename T>
void nn_correct(rtg_handle* h, const float* coef, T* z, cudaStream_t s, const int* stop) {
    NNWs* w = get_nn(h);
    OpView<T> v = nview<T>(h);
    v.stop = stop;
    colstats<T>(h, w, z, false, s, stop);
    nn_correct_kernel<T><<<elem_grid(v.nelem), 256, 0, s>>>(v, coef, w->phi, w->em, w->cm, w->nbr8, w->row_off, z), count_launch();
    RTG_CUDA(cudaGetLastError());
}

template <typename T>
void nn_stats(rtg_handle* h, const T* z, const T* err, const float* scale, float weight, float* S, cudaStream_t s) {
    NNWs* w = get_nn(h);
    const OpView<T>& v = nview<T>(h);
    nn_stats_kernel<T><<<elem_grid(v.nelem), 256, 0, s>>>(v, z, err, w->row_off, scale, weight, S), count_launch();
    RTG_CUDA(cudaGetLastError());
}

int64_t nn_work_floats() { return (int64_t)kGradCtas * kNP + 2 * kGradCtas; }

void nn_loss_grad(const float* params, const float* feat, const float* mom, const float* stats, int64_t rows,
                  float* work, float* grad, double* loss, cudaStream_t s) {
    mlp_attributes();
    const int64_t ntiles = std::max<int64_t>(1, (rows + kTile - 1) / kTile);
    const int grid = (int)std::min<int64_t>(ntiles, kGradCtas);
    double* lossw = reinterpret_cast<double*>(work + (int64_t)kGradCtas * kNP);
    nn_grad_kernel<<<grid, kMlpThreads, kMlpSmem, s>>>(params, feat, mom, stats, std::max<int64_t>(rows, 0), work,
                                                       lossw), count_launch();
    nn_reduce_grad_kernel<<<(kNP + 255) / 256, 256, 0, s>>>(work, grid, lossw, grad, loss), count_launch();
    RTG_CUDA(cudaGetLastError());
}

void nn_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float b1, float b2,
             float eps, float wd, cudaStream_t s) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    nn_adam_kernel<<<(kNP + 255) / 256, 256, 0, s>>>(params, grad, m, v, kNP, lr, b1, b2, eps, wd, c1, c2), count_launch();
    RTG_CUDA(cudaGetLastError());
}

// z += L z with the handle's coefficients (z is the sweep output)
template <typename T>
void apply_learned(rtg_handle* h, T* z, cudaStream_t s, const int* stop) {
    NNWs* w = get_nn(h);
    if (!w->has_params) throw RtgError{RTG_ERR_ARG, "no network set on the handle"};
    nn_correct<T>(h, w->coef, z, s, stop);
}

template void nn_moments<double>(rtg_handle*, const double*, float*, float*, cudaStream_t);
template void nn_moments<float>(rtg_handle*, const float*, float*, float*, cudaStream_t);
template void nn_correct<double>(rtg_handle*, const float*, double*, cudaStream_t, const int*);
template void nn_correct<float>(rtg_handle*, const float*, float*, cudaStream_t, const int*);
template void nn_stats<double>(rtg_handle*, const double*, const double*, const float*, float, float*, cudaStream_t);
template void nn_stats<float>(rtg_handle*, const float*, const float*, const float*, float, float*, cudaStream_t);
template void apply_learned<double>(rtg_handle*, double*, cudaStream_t, const int*);
template void apply_learned<float>(rtg_handle*, float*, cudaStream_t, const int*);

}  // namespace rtg

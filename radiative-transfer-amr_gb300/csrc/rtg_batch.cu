// Batched solve of many independent RT instances held by one handle.
//
// The instances' meshes are concatenated into one mesh description (no
// couplings between instances), so every operator apply and every sweep
// covers all instances in one launch.  The Krylov state is per instance:
// inner products are segmented by instance, the Hessenberg matrix, Givens
// rotations and convergence flags of each instance live on the device and
// are updated by one thread per instance, and a converged instance's basis is
// frozen.  One GMRES restart cycle (m Arnoldi steps, the correction and its
// sweep) is a fixed kernel sequence, captured once in a CUDA graph and
// replayed; the host reads the per-instance flags once per cycle.
//
// method 1 (the batched workload's method): FP64 iterative refinement around
// FP32 sweep-preconditioned GMRES; method 0: FP64 GMRES.
//
// Instances converge at different iterations; a finished instance costs
// nothing for the rest of the cycle: per-column skip flags (refreshed inside
// the captured cycle from the per-instance flags) make the operator apply and
// the sweep leave its columns out, and the vector kernels leave out its
// chunks.  Its frozen basis columns and correction are never read again.
#include <chrono>
#include <cmath>
#include <type_traits>
#include <vector>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kBChunk = 4096;
constexpr int kBThreads = 256;
constexpr int kBGroup = 8;

struct BChunk {
    int64_t begin, end;
    int32_t inst, pad;
};

template <typename T>
__global__ void bdot_kernel(const BChunk* __restrict__ ch, const T* __restrict__ V, int64_t ldv, int k,
                            const T* __restrict__ w, double* __restrict__ partial, const int32_t* __restrict__ done) {
    __shared__ double red[kBGroup][kBThreads / 32];
    const BChunk c = ch[blockIdx.x];
    if (done && done[c.inst]) return;
    for (int g0 = 0; g0 < k; g0 += kBGroup) {
        const int gk = min(kBGroup, k - g0);
        // per element and per warp in the vectors' precision (FP32 stays on
        // the FP32 pipe), double from the per-warp sums on
        T acc[kBGroup];
#pragma unroll
        for (int q = 0; q < kBGroup; ++q) acc[q] = T(0);
        for (int64_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
            const T wi = w[i];
#pragma unroll
            for (int q = 0; q < kBGroup; ++q)
                if (q < gk) acc[q] = fma(V[(int64_t)(g0 + q) * ldv + i], wi, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < kBGroup; ++q) {
            T sw = acc[q];
            for (int o = 16; o > 0; o >>= 1) sw += __shfl_down_sync(0xffffffffu, sw, o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = (double)sw;
        }
        __syncthreads();
        if (threadIdx.x < gk) {
            double s = 0.;
            for (int wq = 0; wq < kBThreads / 32; ++wq) s += red[threadIdx.x][wq];
            partial[(int64_t)blockIdx.x * k + g0 + threadIdx.x] = s;
        }
        __syncthreads();
    }
}

// out[b*ldo + q] = sum of the partials of instance b; with add, also
// out_sum[b*ldo + q] = out + add.
__global__ void breduce_kernel(const int32_t* __restrict__ cbeg, const double* __restrict__ partial, int k,
                               double* __restrict__ out, int ldo, const double* __restrict__ add,
                               double* __restrict__ out_sum) {
    const int b = blockIdx.x, q = blockIdx.y;
    double s = 0.;
    for (int c = cbeg[b] + threadIdx.x; c < cbeg[b + 1]; c += blockDim.x) s += partial[(int64_t)c * k + q];
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.;
        for (int wq = 0; wq < (int)(blockDim.x + 31) / 32; ++wq) t += red[wq];
        out[b * ldo + q] = t;
        if (add) out_sum[b * ldo + q] = t + add[b * ldo + q];
    }
}

// w -= sum_{q<k} h[b][q] V_q on the chunk's instance b
template <typename T>
__global__ void baxpy_kernel(const BChunk* __restrict__ ch, T* __restrict__ w, const T* __restrict__ V, int64_t ldv,
                             int k, const double* __restrict__ h, int ldh, const int32_t* __restrict__ done) {
    __shared__ T hs[64];
    const BChunk c = ch[blockIdx.x];
    if (done && done[c.inst]) return;
    if (threadIdx.x < k) hs[threadIdx.x] = (T)h[c.inst * ldh + threadIdx.x];
    __syncthreads();
    for (int64_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
        T sv = w[i];
        for (int q = 0; q < k; ++q) sv = fma(-hs[q], V[(int64_t)q * ldv + i], sv);
        w[i] = sv;
    }
}

// out = w / sqrt(nsq[b]); hcol[b*ldh + jcol] = sqrt(nsq[b]) (first chunk of b)
template <typename T>
__global__ void bnormalize_kernel(const BChunk* __restrict__ ch, const int32_t* __restrict__ cbeg,
                                  const T* __restrict__ w, T* __restrict__ out, const double* __restrict__ nsq,
                                  int ldn, double* __restrict__ hcol, int ldh, int jcol,
                                  const int32_t* __restrict__ done) {
    const BChunk c = ch[blockIdx.x];
    if (done && done[c.inst]) return;
    const double nr = sqrt(nsq[c.inst * ldn]);
    if (hcol && threadIdx.x == 0 && cbeg[c.inst] == (int)blockIdx.x) hcol[c.inst * ldh + jcol] = nr;
    const T inv = (T)(nr > 0. ? 1. / nr : 0.);
    for (int64_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) out[i] = w[i] * inv;
}

// x += scale[b] * sum_{q < kb[b]} y[b][q] V_q
template <typename TV, typename TX>
__global__ void bcombine_kernel(const BChunk* __restrict__ ch, TX* __restrict__ x, const TV* __restrict__ V,
                                int64_t ldv, const int32_t* __restrict__ kb, const double* __restrict__ y, int ldy) {
    using A = typename std::conditional<sizeof(TV) == 4 && sizeof(TX) == 4, float, double>::type;
    __shared__ A ys[64];
    __shared__ int s_k;
    const BChunk c = ch[blockIdx.x];
    if (threadIdx.x == 0) s_k = kb[c.inst];
    if (threadIdx.x < 64) ys[threadIdx.x] = (A)y[c.inst * ldy + min((int)threadIdx.x, ldy - 1)];
    __syncthreads();
    const int k = s_k;
    for (int64_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
        A sv = A(0);
        for (int q = 0; q < k; ++q) sv = fma(ys[q], (A)V[(int64_t)q * ldv + i], sv);
        x[i] = (TX)((A)x[i] + sv);
    }
}

// y = a[b] * x + beta * y  (a per instance; a == nullptr means ascal); a zero
// coefficient drops its term without reading it (uninitialised buffers)
template <typename TX, typename TY>
__global__ void bscale_kernel(const BChunk* __restrict__ ch, const TX* __restrict__ x, TY* __restrict__ y,
                              const double* __restrict__ a, int lda, double ascal, double beta) {
    using A = typename std::conditional<sizeof(TX) == 4 && sizeof(TY) == 4, float, double>::type;
    const BChunk c = ch[blockIdx.x];
    const double s = a ? a[c.inst * lda] : ascal;
    const A sa = (A)s, ba = (A)beta;
    for (int64_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x)
        y[i] = (TY)((s == 0. ? A(0) : sa * (A)x[i]) + (beta == 0. ? A(0) : ba * (A)y[i]));
}

// Start of a restart cycle, one thread per instance: beta = ||r||, g = (beta, 0...).
__global__ void bstart_kernel(int nb, int m, const double* __restrict__ nsq, int ldn, double* __restrict__ g,
                              const double* __restrict__ tol, int32_t* __restrict__ kvalid,
                              int32_t* __restrict__ done) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const double beta = sqrt(nsq[b * ldn]);
    for (int q = 0; q <= m; ++q) g[b * (m + 1) + q] = 0.;
    g[b * (m + 1)] = beta;
    kvalid[b] = 0;
    done[b] = (beta <= tol[b]) ? 1 : 0;
}

// Arnoldi step j of every instance, one thread per instance: store the new
// Hessenberg column, apply the previous Givens rotations, form the new one,
// update g and the residual estimate; freeze the instance once converged.
__global__ void barnoldi_kernel(int nb, int m, int j, const double* __restrict__ ho, int ldh, double* __restrict__ H,
                                double* __restrict__ cs, double* __restrict__ sn, double* __restrict__ g,
                                const double* __restrict__ tol, int32_t* __restrict__ kvalid,
                                int32_t* __restrict__ done, double* __restrict__ est) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || done[b]) return;
    double* hc = H + (int64_t)b * (m + 1) * m + (int64_t)j * (m + 1);
    for (int q = 0; q <= j + 1; ++q) hc[q] = ho[b * ldh + q];
    double* c = cs + b * m;
    double* s = sn + b * m;
    for (int q = 0; q < j; ++q) {
        const double a0 = hc[q], a1 = hc[q + 1];
        hc[q] = c[q] * a0 + s[q] * a1;
        hc[q + 1] = -s[q] * a0 + c[q] * a1;
    }
    const double a0 = hc[j], a1 = hc[j + 1];
    const double rr = hypot(a0, a1);
    c[j] = rr > 0. ? a0 / rr : 1.;
    s[j] = rr > 0. ? a1 / rr : 0.;
    hc[j] = rr;
    hc[j + 1] = 0.;
    double* gg = g + b * (m + 1);
    gg[j + 1] = -s[j] * gg[j];
    gg[j] = c[j] * gg[j];
    const double e = fabs(gg[j + 1]);
    est[b] = e;
    kvalid[b] = j + 1;
    if (e <= tol[b] || rr == 0. || !isfinite(e)) done[b] = 1;
}

// y = H^{-1} g on the kvalid columns of each instance (back substitution)
__global__ void bsolve_kernel(int nb, int m, const double* __restrict__ H, const double* __restrict__ g,
                              const int32_t* __restrict__ kvalid, double* __restrict__ y) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int k = kvalid[b];
    const double* Hb = H + (int64_t)b * (m + 1) * m;
    double* yb = y + b * m;
    for (int q = k - 1; q >= 0; --q) {
        double acc = g[b * (m + 1) + q];
        for (int cc = q + 1; cc < k; ++cc) acc -= Hb[(int64_t)cc * (m + 1) + q] * yb[cc];
        const double d = Hb[(int64_t)q * (m + 1) + q];
        yb[q] = d != 0. ? acc / d : 0.;
    }
    for (int q = k; q < m; ++q) yb[q] = 0.;
}

// Per-column skip flags from the per-instance state: mode 0 skips finished
// instances (done), mode 1 skips instances without a correction (kvalid 0).
__global__ void bskip_kernel(int ncols, const int32_t* __restrict__ col_inst, const int32_t* __restrict__ done,
                             const int32_t* __restrict__ kvalid, int mode, int32_t* __restrict__ skip) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    const int b = col_inst[c];
    skip[c] = mode == 0 ? (done[b] != 0) : (kvalid[b] == 0);
}

// d += z on the chunks of instances that formed a correction this cycle
__global__ void badd_kernel(const BChunk* __restrict__ ch, const float* __restrict__ z, float* __restrict__ d,
                            const int32_t* __restrict__ kvalid) {
    const BChunk c = ch[blockIdx.x];
    if (kvalid[c.inst] == 0) return;
    for (int64_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) d[i] += z[i];
}

inline int grid1(int n) { return (n + 127) / 128; }

}  // namespace

struct BatchWs {
    int nb = 0, m = 0, nchunks = 0;
    int64_t N = 0;
    BChunk* d_ch = nullptr;
    int32_t* d_cbeg = nullptr;
    double *b = nullptr, *r = nullptr, *x = nullptr, *t = nullptr, *gb = nullptr;
    float *V32 = nullptr, *w32 = nullptr, *z32 = nullptr, *s32 = nullptr, *d32 = nullptr, *rhs32 = nullptr;
    double *partial = nullptr, *h1 = nullptr, *h2 = nullptr, *ho = nullptr, *nsq = nullptr;
    double *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr, *est = nullptr;
    double *tol = nullptr, *tin = nullptr, *scale = nullptr, *vnorm = nullptr;
    int32_t *kvalid = nullptr, *done = nullptr;
    int32_t *col_inst = nullptr, *col_skip = nullptr;   // per column: instance, skip flag
    cudaGraphExec_t cycle = nullptr;
    long long cycle_kernels = 0;   // kernels one replay of the cycle runs
    std::vector<void*> allocs;
};

namespace {

template <typename T>
T* balloc(BatchWs* w, size_t n) {
    void* p = nullptr;
    RTG_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)));
    w->allocs.push_back(p);
    return (T*)p;
}

void free_bws(BatchWs* w) {
    if (!w) return;
    if (w->cycle) cudaGraphExecDestroy(w->cycle);
    for (void* p : w->allocs) cudaFree(p);
    delete w;
}

// per-instance squared norms into out[b*ldo]
template <typename T>
void bnorm2(const BatchWs* w, const T* v, double* out, int ldo, cudaStream_t s, const int32_t* done = nullptr) {
    bdot_kernel<T><<<w->nchunks, kBThreads, 0, s>>>(w->d_ch, v, 0, 1, v, w->partial, done), count_launch();
    breduce_kernel<<<dim3(w->nb, 1), 128, 0, s>>>(w->d_cbeg, w->partial, 1, out, ldo, nullptr, nullptr), count_launch();
}

// One restart cycle of batched FP32 GMRES for A d = rhs32, sweep right
// preconditioned, d updated in place; the kernel sequence is fixed.
void record_cycle(rtg_handle* h, BatchWs* w, cudaStream_t s) {
    const int m = w->m, nb = w->nb, nc = w->nchunks;
    const int64_t N = w->N;
    const int ldh = m + 2;
    const int ncols = h->v32.ncols;
    OpView<float> v = h->v32;       // the operator with the batch's column skip flags
    v.skip = w->col_skip;
    // w = rhs - A d ; V0 = w / ||w|| ; start
    launch_apply<float>(h, h->v32, RTG_SYSTEM | RTG_MASK_ROWS, w->d32, w->s32, s);
    bscale_kernel<float, float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->rhs32, w->w32, nullptr, 0, 1., 0.), count_launch();
    bscale_kernel<float, float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->s32, w->w32, nullptr, 0, -1., 1.), count_launch();
    bnorm2<float>(w, w->w32, w->nsq, 1, s);
    bnormalize_kernel<float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->d_cbeg, w->w32, w->V32, w->nsq, 1, nullptr, 0, 0,
                                                      nullptr), count_launch();
    bstart_kernel<<<grid1(nb), 128, 0, s>>>(nb, m, w->nsq, 1, w->g, w->tin, w->kvalid, w->done), count_launch();
    for (int j = 0; j < m; ++j) {
        float* vj = w->V32 + (int64_t)j * N;
        float* vn = w->V32 + (int64_t)(j + 1) * N;
        bskip_kernel<<<grid1(ncols), 128, 0, s>>>(ncols, w->col_inst, w->done, w->kvalid, 0, w->col_skip), count_launch();
        apply_sweep<float>(h, vj, w->z32, s, nullptr, w->col_skip);
        launch_apply<float>(h, v, RTG_SYSTEM | RTG_MASK_ROWS, w->z32, w->w32, s);
        // CGS2 with per-instance coefficients; ho = h1 + h2
        bdot_kernel<float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->V32, N, j + 1, w->w32, w->partial, w->done), count_launch();
        breduce_kernel<<<dim3(nb, j + 1), 128, 0, s>>>(w->d_cbeg, w->partial, j + 1, w->h1, ldh, nullptr, nullptr), count_launch();
        baxpy_kernel<float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->w32, w->V32, N, j + 1, w->h1, ldh, w->done), count_launch();
        bdot_kernel<float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->V32, N, j + 1, w->w32, w->partial, w->done), count_launch();
        breduce_kernel<<<dim3(nb, j + 1), 128, 0, s>>>(w->d_cbeg, w->partial, j + 1, w->h2, ldh, w->h1, w->ho), count_launch();
        baxpy_kernel<float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->w32, w->V32, N, j + 1, w->h2, ldh, w->done), count_launch();
        bnorm2<float>(w, w->w32, w->nsq, 1, s, w->done);
        bnormalize_kernel<float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->d_cbeg, w->w32, vn, w->nsq, 1, w->ho, ldh, j + 1,
                                                          w->done), count_launch();
        barnoldi_kernel<<<grid1(nb), 128, 0, s>>>(nb, m, j, w->ho, ldh, w->H, w->cs, w->sn, w->g, w->tin, w->kvalid,
                                                   w->done, w->est), count_launch();
    }
    // d += P^{-1} (V y), for the instances that formed a correction
    bsolve_kernel<<<grid1(nb), 128, 0, s>>>(nb, m, w->H, w->g, w->kvalid, w->y), count_launch();
    bscale_kernel<float, float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->s32, w->s32, nullptr, 0, 0., 0.), count_launch();
    bcombine_kernel<float, float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->s32, w->V32, N, w->kvalid, w->y, m), count_launch();
    bskip_kernel<<<grid1(ncols), 128, 0, s>>>(ncols, w->col_inst, w->done, w->kvalid, 1, w->col_skip), count_launch();
    apply_sweep<float>(h, w->s32, w->z32, s, nullptr, w->col_skip);
    badd_kernel<<<nc, kBThreads, 0, s>>>(w->d_ch, w->z32, w->d32, w->kvalid), count_launch();
}

}  // namespace

void free_batch(rtg_handle* h) {
    free_bws(h->bws);
    h->bws = nullptr;
}

int solve_batched(rtg_handle* h, int nb, const int64_t* inst_off, const double* f, const double* g, double* u,
                  const rtg_solve_opts* o, rtg_solve_info* infos, cudaStream_t s) {
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t N = h->host.ndof;
    if (nb < 1) throw RtgError{RTG_ERR_ARG, "nbatch < 1"};
    if (inst_off[0] != 0 || inst_off[nb] != N) throw RtgError{RTG_ERR_ARG, "instance offsets must cover [0, N)"};
    for (int b = 0; b < nb; ++b)
        if (inst_off[b + 1] <= inst_off[b]) throw RtgError{RTG_ERR_ARG, "empty or unordered instance"};
    if (o->method != 1) throw RtgError{RTG_ERR_ARG, "batched solve supports method 1 (FP32 GMRES + FP64 refinement)"};
    const int m = std::max(1, std::min(o->restart, 60));
    get_sweep(h, s);
    // (re)build the workspace when the instance split or restart changes
    BatchWs* w = h->bws;
    bool same = w && w->nb == nb && w->m == m && w->N == N;
    std::vector<BChunk> chunks;
    std::vector<int32_t> cbeg(nb + 1, 0);
    for (int b = 0; b < nb; ++b) {
        cbeg[b] = (int32_t)chunks.size();
        for (int64_t i = inst_off[b]; i < inst_off[b + 1]; i += kBChunk)
            chunks.push_back(BChunk{i, std::min(inst_off[b + 1], i + kBChunk), b, 0});
    }
    cbeg[nb] = (int32_t)chunks.size();
    if (same) {
        std::vector<int32_t> old(nb + 1);
        RTG_CUDA(cudaMemcpy(old.data(), w->d_cbeg, sizeof(int32_t) * (nb + 1), cudaMemcpyDeviceToHost));
        same = old == cbeg;
    }
    if (!same) {
        free_bws(w);
        w = new BatchWs();
        h->bws = w;
        w->nb = nb;
        w->m = m;
        w->N = N;
        w->nchunks = (int)chunks.size();
        w->d_ch = balloc<BChunk>(w, chunks.size());
        w->d_cbeg = balloc<int32_t>(w, nb + 1);
        RTG_CUDA(cudaMemcpy(w->d_ch, chunks.data(), sizeof(BChunk) * chunks.size(), cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemcpy(w->d_cbeg, cbeg.data(), sizeof(int32_t) * (nb + 1), cudaMemcpyHostToDevice));
        w->b = balloc<double>(w, N);
        w->r = balloc<double>(w, N);
        w->x = balloc<double>(w, N);
        w->t = balloc<double>(w, N);
        w->gb = balloc<double>(w, N);
        w->V32 = balloc<float>(w, (size_t)(m + 1) * N);
        w->w32 = balloc<float>(w, N);
        w->z32 = balloc<float>(w, N);
        w->s32 = balloc<float>(w, N);
        w->d32 = balloc<float>(w, N);
        w->rhs32 = balloc<float>(w, N);
        w->partial = balloc<double>(w, (size_t)chunks.size() * (m + 2));
        const int ldh = m + 2;
        w->h1 = balloc<double>(w, (size_t)nb * ldh);
        w->h2 = balloc<double>(w, (size_t)nb * ldh);
        w->ho = balloc<double>(w, (size_t)nb * ldh);
        w->nsq = balloc<double>(w, nb);
        w->H = balloc<double>(w, (size_t)nb * (m + 1) * m);
        w->cs = balloc<double>(w, (size_t)nb * m);
        w->sn = balloc<double>(w, (size_t)nb * m);
        w->g = balloc<double>(w, (size_t)nb * (m + 1));
        w->y = balloc<double>(w, (size_t)nb * m);
        w->est = balloc<double>(w, nb);
        w->tol = balloc<double>(w, nb);
        w->tin = balloc<double>(w, nb);
        w->scale = balloc<double>(w, nb);
        w->vnorm = balloc<double>(w, nb);
        w->kvalid = balloc<int32_t>(w, nb);
        w->done = balloc<int32_t>(w, nb);
        // instance of every column (columns are contiguous in DOF order)
        const HostTables& t = h->host;
        std::vector<int32_t> ci(t.cols.size());
        int b = 0;
        for (size_t c = 0; c < t.cols.size(); ++c) {
            while (b + 1 < nb && t.cols[c].dof_off >= inst_off[b + 1]) ++b;
            if (t.cols[c].dof_off < inst_off[b] || t.cols[c].dof_off + t.cols[c].ndof > inst_off[b + 1])
                throw RtgError{RTG_ERR_ARG, "an instance boundary splits a column"};
            ci[c] = b;
        }
        w->col_inst = balloc<int32_t>(w, ci.size());
        w->col_skip = balloc<int32_t>(w, ci.size());
        RTG_CUDA(cudaMemcpy(w->col_inst, ci.data(), sizeof(int32_t) * ci.size(), cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMemset(w->col_skip, 0, sizeof(int32_t) * ci.size()));
    }
    const int nc = w->nchunks;
    // b = mask_I (f - A mask_B g); x = 0
    launch_mask_vector(h, 1, g, w->gb, s);
    launch_apply<double>(h, h->v64, RTG_SYSTEM | RTG_MASK_ROWS, w->gb, w->t, s);
    launch_mask_vector(h, 0, f, w->b, s);
    bscale_kernel<double, double><<<nc, kBThreads, 0, s>>>(w->d_ch, w->t, w->b, nullptr, 0, -1., 1.), count_launch();
    bscale_kernel<double, double><<<nc, kBThreads, 0, s>>>(w->d_ch, w->t, w->x, nullptr, 0, 0., 0.), count_launch();
    std::vector<double> bn(nb), rn(nb), tol(nb), tin(nb), scale(nb), inv(nb);
    bnorm2<double>(w, w->b, w->vnorm, 1, s);
    RTG_CUDA(cudaMemcpyAsync(bn.data(), w->vnorm, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    RTG_CUDA(cudaStreamSynchronize(s));
    for (int b = 0; b < nb; ++b) tol[b] = std::max(o->rtol * std::sqrt(bn[b]), o->atol);
    const double inner_rtol = o->inner_rtol > 0. ? o->inner_rtol : 1e-6;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 20;
    const int max_cycles = std::max(1, o->max_it / m);
    std::vector<int> iters(nb, 0), outer(nb, 0), done(nb), kv(nb), conv(nb, 0);
    int fp64_applies = 1, fp32_applies = 0, sweeps = 0;
    for (int it = 0; it <= max_outer; ++it) {
        // r = b - A x (FP64), per-instance norms
        launch_apply<double>(h, h->v64, RTG_SYSTEM | RTG_MASK_ROWS, w->x, w->r, s);
        ++fp64_applies;
        bscale_kernel<double, double><<<nc, kBThreads, 0, s>>>(w->d_ch, w->b, w->r, nullptr, 0, 1., -1.), count_launch();
        bnorm2<double>(w, w->r, w->vnorm, 1, s);
        RTG_CUDA(cudaMemcpyAsync(rn.data(), w->vnorm, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
        RTG_CUDA(cudaStreamSynchronize(s));
        bool any = false;
        for (int b = 0; b < nb; ++b) {
            rn[b] = std::sqrt(rn[b]);
            const bool act = rn[b] > tol[b] && std::isfinite(rn[b]);
            conv[b] = act ? 0 : 1;
            any = any || act;
            inv[b] = act ? 1. / rn[b] : 0.;
            scale[b] = act ? rn[b] : 0.;
            tin[b] = act ? std::max(inner_rtol, tol[b] / rn[b]) : 1e300;
            if (act) outer[b]++;
        }
        if (!any || it == max_outer) break;
        // inner FP32 solve of A d = r / ||r|| per instance
        RTG_CUDA(cudaMemcpyAsync(w->scale, inv.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, s));
        RTG_CUDA(cudaMemcpyAsync(w->tin, tin.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, s));
        bscale_kernel<double, float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->r, w->rhs32, w->scale, 1, 0., 0.), count_launch();
        bscale_kernel<float, float><<<nc, kBThreads, 0, s>>>(w->d_ch, w->d32, w->d32, nullptr, 0, 0., 0.), count_launch();
        if (!w->cycle) {
            // build the FP32 apply plan and sweep launch shape before capture
            launch_apply<float>(h, h->v32, RTG_SYSTEM | RTG_MASK_ROWS, w->d32, w->s32, s);
            apply_sweep<float>(h, w->s32, w->z32, s);
            RTG_CUDA(cudaStreamSynchronize(s));
            cudaStream_t cap;
            RTG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            cudaGraph_t graph;
            const long long n0 = launch_counter().load();
            RTG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            record_cycle(h, w, cap);
            RTG_CUDA(cudaStreamEndCapture(cap, &graph));
            // recorded launches are counted when the graph runs
            w->cycle_kernels = launch_counter().load() - n0;
            launch_counter().fetch_sub(w->cycle_kernels);
            RTG_CUDA(cudaGraphInstantiate(&w->cycle, graph, 0));
            RTG_CUDA(cudaGraphDestroy(graph));
            RTG_CUDA(cudaStreamDestroy(cap));
        }
        for (int cyc = 0; cyc < max_cycles; ++cyc) {
            RTG_CUDA(cudaGraphLaunch(w->cycle, s));
            launch_counter().fetch_add(w->cycle_kernels);
            fp32_applies += m + 1;
            sweeps += m + 1;
            RTG_CUDA(cudaMemcpyAsync(done.data(), w->done, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
            RTG_CUDA(cudaMemcpyAsync(kv.data(), w->kvalid, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
            RTG_CUDA(cudaStreamSynchronize(s));
            bool all = true;
            for (int b = 0; b < nb; ++b) {
                if (!conv[b]) iters[b] += kv[b];
                all = all && (done[b] || conv[b]);
            }
            if (all) break;
        }
        // x += ||r|| d
        RTG_CUDA(cudaMemcpyAsync(w->scale, scale.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, s));
        bscale_kernel<float, double><<<nc, kBThreads, 0, s>>>(w->d_ch, w->d32, w->x, w->scale, 1, 0., 1.), count_launch();
    }
    if (sweep_status(h, s) != RTG_OK)
        throw RtgError{RTG_ERR_TIMEOUT, "a sweep wait gave up; the solution is not valid"};
    // u = x on the unknowns, g on the inflow-boundary DOFs
    bscale_kernel<double, double><<<nc, kBThreads, 0, s>>>(w->d_ch, w->x, w->gb, nullptr, 0, 1., 1.), count_launch();
    RTG_CUDA(cudaMemcpyAsync(u, w->gb, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    RTG_CUDA(cudaStreamSynchronize(s));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (infos)
        for (int b = 0; b < nb; ++b) {
            rtg_solve_info inf{};
            inf.converged = conv[b];
            inf.iterations = iters[b];
            inf.outer = outer[b];
            inf.fp64_applies = fp64_applies;
            inf.fp32_applies = fp32_applies;
            inf.sweeps = sweeps;
            inf.res_f = rn[b];
            inf.rhs_norm = std::sqrt(bn[b]);
            inf.seconds = secs;
            infos[b] = inf;
        }
    return RTG_OK;
}

}  // namespace rtg

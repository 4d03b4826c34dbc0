// Two-level preconditioner: the upwind sweep followed by a diffusion
// correction on the spatial columns (diffusion synthetic acceleration used as
// the coarse level of a multiplicative two-level preconditioner).
//
// The sweep (rtg_sweep.cu) inverts streaming and extinction.  What it leaves
// is the error that scattering spreads over directions and space; in optically
// thick, highly scattering regions that error is smooth in space and close to
// isotropic, a diffusion mode, and no sweep-sized correction removes it.  The
// coarse level solves for that mode: with the residual r = v - A z of the
// sweep output z, the angle-integrated error equation with the P1 closure in
// the plane,
//     -div( D grad Phi ) + sigma_a Phi = int r dth,   D = 1 / (2 sigma_tr),
// is discretised cell-centred on the columns: one unknown Phi_C per column,
// sigma_a = sigma_t - sigma_s and sigma_tr = sigma_t - gbar sigma_s from the
// column means of kappa and sigma (gbar: the mean scattering cosine of the
// column's discrete phase-function matrix), two-point face fluxes
// |f| (Phi_C - Phi_N) / (d_C / D_C + d_N / D_N) (d: centre-to-face distances;
// a face to two finer neighbours gives two sub-faces) and, on faces without a
// neighbour, the vacuum (Marshak) flux |f| Phi_C / (d_C / D_C + pi / 2).  The
// right-hand side of column C is the sum of the weak-form residual over the
// column's unknowns (the DG residual already carries the quadrature weights),
// and the correction adds the isotropic angular flux Phi_C / (2 pi) to the
// column's unknowns:
//     z = P_sweep^{-1} v;  r = v - A z;  z += P D_c^{-1} R r.
// D_c (ncols x ncols, symmetric, diagonally dominant) is inverted once,
// densely, by Gauss-Jordan elimination with partial pivoting in FP64 on the
// device; each application is then one dense matrix-vector product.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kMaxCoarse = 24000;  // dense coarse operator: 16 n^2 bytes, 2 n^3 FP64 FMA to invert
constexpr double kPiC = 3.141592653589793;

__device__ __forceinline__ bool bdry_node_c(int bm, int i, int j, int nx, int ny) {
    return ((bm & 1) && i == nx - 1) || ((bm & 2) && j == ny - 1) || ((bm & 4) && i == 0) ||
           ((bm & 8) && j == 0);
}

// out[C] = sum of y over the unknowns of column C (one CTA per column, FP64)
template <typename T>
__global__ void restrict_kernel(OpView<T> v, const T* __restrict__ y, double* __restrict__ out) {
    __shared__ double red[32];
    const int ci = blockIdx.x;
    const ColDev C = v.cols[ci];
    const int nij = C.nx * C.ny;
    double acc = 0.;
    for (int e = C.elem_begin; e < C.elem_end; ++e) {
        const ElemDev E = v.elems[e];
        const int nth = E.nth, bm = E.flags >> 4;
        for (int l = threadIdx.x; l < nij * nth; l += blockDim.x) {
            const int ij = l / nth, i = ij / C.ny, j = ij % C.ny;
            if (bdry_node_c(bm, i, j, C.nx, C.ny)) continue;
            acc += (double)y[E.dof_off + l];
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s += red[w];
        out[ci] = s;
    }
}

// z += c[C] / (2 pi) at the unknowns of every column C (one warp per element)
template <typename T, typename TC>
__global__ void prolong_kernel(OpView<T> v, const TC* __restrict__ c, T* __restrict__ z) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < v.nelem; e += gridDim.x * wpb) {
        const ElemDev E = v.elems[e];
        const ColDev C = v.cols[E.col];
        const int nth = E.nth, bm = E.flags >> 4;
        const T add = (T)((double)c[E.col] * (0.5 / kPiC));
        for (int ij = lane; ij < C.nx * C.ny; ij += 32) {
            const int i = ij / C.ny, j = ij % C.ny;
            if (bdry_node_c(bm, i, j, C.nx, C.ny)) continue;
            T* ze = z + E.dof_off + (int64_t)ij * nth;
            for (int a = 0; a < nth; ++a) ze[a] += add;
        }
    }
}

// y = M x for a dense n x n row-major M (one warp per row)
template <typename TM>
__global__ void gemv_kernel(const TM* __restrict__ M, const double* __restrict__ x, int n, TM* __restrict__ y) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int r = blockIdx.x * wpb + (threadIdx.x >> 5); r < n; r += gridDim.x * wpb) {
        const TM* row = M + (int64_t)r * n;
        double s = 0.;
        for (int c = lane; c < n; c += 32) s += (double)row[c] * x[c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) y[r] = (TM)s;
    }
}

template <typename T>
__global__ void residual_kernel(const T* __restrict__ v, T* __restrict__ r, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = v[i] - r[i];
}

// ---------------------------------------------------------- Gauss-Jordan
// Dense [M | I] of n rows and 2n columns, row-major, FP64.
__global__ void gj_pivot_kernel(const double* __restrict__ M, int n, int k, int* __restrict__ piv,
                                double* __restrict__ pval, int* __restrict__ status) {
    __shared__ double bv[32];
    __shared__ int bi[32];
    const int ld = 2 * n;
    double best = -1.;
    int arg = k;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
        const double a = fabs(M[(int64_t)i * ld + k]);
        if (a > best) {
            best = a;
            arg = i;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, arg, o);
        if (ov > best || (ov == best && oi < arg)) {
            best = ov;
            arg = oi;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        bv[threadIdx.x >> 5] = best;
        bi[threadIdx.x >> 5] = arg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x + 31) / 32; ++w)
            if (bv[w] > best || (bv[w] == best && bi[w] < arg)) {
                best = bv[w];
                arg = bi[w];
            }
        *piv = arg;
        *pval = M[(int64_t)arg * ld + k];
        if (!(best > 0.)) *status = 1;
    }
}

// fcol[i] = entry (i, k) of the matrix after rows k and piv are swapped (read
// before the swap kernel runs)
__global__ void gj_column_kernel(const double* __restrict__ M, int n, int k, const int* __restrict__ piv,
                                 double* __restrict__ fcol) {
    const int ld = 2 * n, p = *piv;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int src = i == k ? p : (i == p ? k : i);
        fcol[i] = M[(int64_t)src * ld + k];
    }
}

// swap rows k and piv, scale row k by 1/pivot (each thread owns one column)
__global__ void gj_swap_scale_kernel(double* __restrict__ M, int n, int k, const int* __restrict__ piv,
                                     const double* __restrict__ pval) {
    const int ld = 2 * n, p = *piv;
    const double inv = *pval != 0. ? 1. / *pval : 0.;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ld; j += gridDim.x * blockDim.x) {
        const double a = M[(int64_t)k * ld + j], b = M[(int64_t)p * ld + j];
        M[(int64_t)p * ld + j] = a;
        M[(int64_t)k * ld + j] = b * inv;
    }
}

// M[i][j] -= fcol[i] * M[k][j] for i != k, j in [k, 2n)
__global__ void gj_eliminate_kernel(double* __restrict__ M, int n, int k, const double* __restrict__ fcol) {
    const int ld = 2 * n;
    const int i = blockIdx.y;
    if (i == k) return;
    const double f = fcol[i];
    if (f == 0.) return;
    const double* rk = M + (int64_t)k * ld;
    double* ri = M + (int64_t)i * ld;
    for (int j = k + blockIdx.x * blockDim.x + threadIdx.x; j < ld; j += gridDim.x * blockDim.x)
        ri[j] -= f * rk[j];
}

__global__ void gj_identity_kernel(double* __restrict__ M, int n) {
    const int64_t nn = (int64_t)n * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / n, j = t % n;
        M[i * 2 * n + n + j] = i == j ? 1. : 0.;
    }
}

__global__ void gj_extract_kernel(const double* __restrict__ M, int n, double* __restrict__ inv64,
                                  float* __restrict__ inv32) {
    const int64_t nn = (int64_t)n * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / n, j = t % n;
        const double val = M[i * 2 * n + n + j];
        inv64[t] = val;
        inv32[t] = (float)val;
    }
}

inline int egrid(int n) { return std::max(1, std::min((n + 7) / 8, 152 * 16)); }
inline int vgrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

template <typename T>
const OpView<T>& cview(const rtg_handle* h);
template <>
const OpView<double>& cview<double>(const rtg_handle* h) { return h->v64; }
template <>
const OpView<float>& cview<float>(const rtg_handle* h) { return h->v32; }

// Dense inverse of the n x n row-major host matrix A on the device.
void invert_dense(const std::vector<double>& A, int n, double* inv64, float* inv32, cudaStream_t s) {
    double *M = nullptr, *small = nullptr, *fcol = nullptr;
    auto release = [&] {
        for (double* p : {M, small, fcol})
            if (p) cudaFree(p);
    };
    try {
        RTG_CUDA(cudaMalloc(&M, sizeof(double) * (size_t)n * 2 * n));
        RTG_CUDA(cudaMalloc(&small, sizeof(double) * 4));
        RTG_CUDA(cudaMalloc(&fcol, sizeof(double) * n));
        RTG_CUDA(cudaMemcpy2DAsync(M, sizeof(double) * 2 * n, A.data(), sizeof(double) * n, sizeof(double) * n, n,
                                   cudaMemcpyHostToDevice, s));
        gj_identity_kernel<<<vgrid((int64_t)n * n), 256, 0, s>>>(M, n), count_launch();
        int* dpiv = (int*)small;
        double* dpval = small + 1;
        int* dstatus = (int*)(small + 2);
        RTG_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
        for (int k = 0; k < n; ++k) {
            gj_pivot_kernel<<<1, 1024, 0, s>>>(M, n, k, dpiv, dpval, dstatus), count_launch();
            gj_column_kernel<<<std::max(1, std::min((n + 255) / 256, 256)), 256, 0, s>>>(M, n, k, dpiv, fcol), count_launch();
            gj_swap_scale_kernel<<<std::max(1, std::min((2 * n + 255) / 256, 1024)), 256, 0, s>>>(M, n, k, dpiv,
                                                                                                   dpval), count_launch();
            dim3 g(std::max(1, std::min((2 * n - k + 255) / 256, 8)), n);
            gj_eliminate_kernel<<<g, 256, 0, s>>>(M, n, k, fcol), count_launch();
        }
        gj_extract_kernel<<<vgrid((int64_t)n * n), 256, 0, s>>>(M, n, inv64, inv32), count_launch();
        int status = 0;
        RTG_CUDA(cudaMemcpyAsync(&status, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
        RTG_CUDA(cudaStreamSynchronize(s));
        RTG_CUDA(cudaGetLastError());
        if (status) throw RtgError{RTG_ERR_NONFINITE, "coarse diffusion operator is singular"};
    } catch (...) {
        release();
        throw;
    }
    release();
}

}  // namespace

struct Coarse {
    int n = 0;                    // coarse unknowns (one per column)
    double* inv64 = nullptr;      // [n][n]
    float* inv32 = nullptr;
    double* bc = nullptr;         // [n] restricted residual
    double* cc64 = nullptr;       // [n] coarse solution
    float* cc32 = nullptr;
    double* r64 = nullptr;        // [N] residual work vector
    float* r32 = nullptr;
    std::vector<double> Dc;       // the assembled operator (host, row-major)
    std::vector<void*> allocs;
};

static void* c_alloc(Coarse* c, size_t bytes) {
    void* p = nullptr;
    RTG_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
    c->allocs.push_back(p);
    return p;
}

void free_coarse(rtg_handle* h) {
    if (!h->coarse) return;
    for (void* p : h->coarse->allocs) cudaFree(p);
    delete h->coarse;
    h->coarse = nullptr;
}

// Mean scattering cosine of each signature's discrete phase-function matrix:
// sum_{R,c} W[R][c] cos(th_R - th_c) / sum_{R,c} W[R][c].
static std::vector<double> mean_cosines(const HostTables& t) {
    const int nsig = (int)t.sig_nth.size();
    std::vector<double> g(nsig, 0.);
    std::vector<int> col_of(nsig, -1);
    for (int ci = 0; ci < (int)t.cols.size(); ++ci)
        if (col_of[t.cols[ci].sig] < 0) col_of[t.cols[ci].sig] = ci;
    for (int s = 0; s < nsig; ++s) {
        const int ci = col_of[s];
        if (ci < 0) continue;
        const ColDev& C = t.cols[ci];
        std::vector<double> cs, sn;
        for (int e = C.elem_begin; e < C.elem_end; ++e) {
            const ElemDev& E = t.elems[e];
            const double* A = &t.ang[E.ang];
            for (int a = 0; a < E.nth; ++a) {
                cs.push_back(A[3 * E.nth + a]);
                sn.push_back(A[4 * E.nth + a]);
            }
        }
        const int m = C.nth_col;
        const double* W = &t.W[t.W_off[s]];
        double num = 0., den = 0.;
        for (int R = 0; R < m; ++R)
            for (int c = 0; c < m; ++c) {
                const double w = W[(size_t)R * m + c];
                num += w * (cs[R] * cs[c] + sn[R] * sn[c]);
                den += w;
            }
        g[s] = den > 0. ? num / den : 0.;
    }
    return g;
}

// Assemble the column diffusion operator and invert it on the device.
void build_coarse(rtg_handle* h, cudaStream_t s) {
    const HostTables& t = h->host;
    const int nc = (int)t.cols.size();
    const int64_t N = t.ndof;
    if (nc > kMaxCoarse) throw RtgError{RTG_ERR_SIZE, "too many columns for the dense coarse operator"};
    Coarse* c = h->coarse;
    if (!c) {
        c = new Coarse();
        h->coarse = c;
        try {
            c->n = nc;
            c->inv64 = (double*)c_alloc(c, sizeof(double) * (size_t)nc * nc);
            c->inv32 = (float*)c_alloc(c, sizeof(float) * (size_t)nc * nc);
            c->bc = (double*)c_alloc(c, sizeof(double) * nc);
            c->cc64 = (double*)c_alloc(c, sizeof(double) * nc);
            c->cc32 = (float*)c_alloc(c, sizeof(float) * nc);
            c->r64 = (double*)c_alloc(c, sizeof(double) * N);
            c->r32 = (float*)c_alloc(c, sizeof(float) * N);
        } catch (...) {
            free_coarse(h);
            throw;
        }
    }
    // column means of sigma_t (kappa) and sigma_s: the node tables hold
    // wx wy kappa and wx wy sigma, and sum wx wy = 4
    const std::vector<double> gbar = mean_cosines(t);
    std::vector<double> D(nc), sa(nc);
    for (int ci = 0; ci < nc; ++ci) {
        const ColDev& C = t.cols[ci];
        double k = 0., sg = 0.;
        for (int q = 0; q < C.nx * C.ny; ++q) {
            k += t.kw[C.node_off + q];
            sg += t.sw[C.node_off + q];
        }
        k *= 0.25;
        sg *= 0.25;
        const double str = std::max(k - gbar[C.sig] * sg, 1e-8 * std::max(k, 1e-300) + 1e-12);
        D[ci] = 0.5 / str;
        sa[ci] = std::max(k - sg, 0.);
    }
    std::vector<double>& Dc = c->Dc;
    Dc.assign((size_t)nc * nc, 0.);
    for (int ci = 0; ci < nc; ++ci) {
        const ColDev& C = t.cols[ci];
        Dc[(size_t)ci * nc + ci] += sa[ci] * C.dx * C.dy;
        for (int F = 0; F < 4; ++F) {
            const int n0 = t.col_nbr_raw[8 * ci + 2 * F], n1 = t.col_nbr_raw[8 * ci + 2 * F + 1];
            const bool xface = F % 2 == 0;
            const double dC = 0.5 * (xface ? C.dx : C.dy);
            if (n0 < 0 && n1 < 0) {
                const double len = xface ? C.dy : C.dx;
                Dc[(size_t)ci * nc + ci] += len / (dC / D[ci] + 0.5 * kPiC);
                continue;
            }
            for (int q = 0; q < 2; ++q) {
                const int nb = q == 0 ? n0 : n1;
                if (nb < 0 || (q == 1 && n1 == n0)) continue;
                const ColDev& Nc = t.cols[nb];
                const double len = std::min(xface ? C.dy : C.dx, xface ? Nc.dy : Nc.dx);
                const double dN = 0.5 * (xface ? Nc.dx : Nc.dy);
                const double tau = len / (dC / D[ci] + dN / D[nb]);
                Dc[(size_t)ci * nc + ci] += tau;
                Dc[(size_t)ci * nc + nb] -= tau;
            }
        }
    }
    invert_dense(Dc, nc, c->inv64, c->inv32, s);
}

int coarse_size(rtg_handle* h) { return h->coarse ? h->coarse->n : 0; }

void coarse_operator(rtg_handle* h, double* out) {
    if (!h->coarse) throw RtgError{RTG_ERR_ARG, "coarse correction not built"};
    std::copy(h->coarse->Dc.begin(), h->coarse->Dc.end(), out);
}

// z += P D_c^{-1} R (v - A z)   (z holds the sweep output of v)
template <typename T>
void apply_coarse(rtg_handle* h, const T* v, T* z, cudaStream_t s) {
    Coarse* c = h->coarse;
    if (!c) throw RtgError{RTG_ERR_ARG, "coarse correction not built"};
    const OpView<T>& ov = cview<T>(h);
    const int64_t N = h->host.ndof;
    T* r = sizeof(T) == 8 ? (T*)c->r64 : (T*)c->r32;
    launch_apply<T>(h, ov, RTG_SYSTEM | RTG_MASK_ROWS, z, r, s);
    residual_kernel<T><<<vgrid(N), 256, 0, s>>>(v, r, N), count_launch();
    restrict_kernel<T><<<ov.ncols, 128, 0, s>>>(ov, r, c->bc), count_launch();
    if (sizeof(T) == 8) {
        gemv_kernel<double><<<egrid(c->n), 256, 0, s>>>(c->inv64, c->bc, c->n, c->cc64), count_launch();
        prolong_kernel<T, double><<<egrid(ov.nelem), 256, 0, s>>>(ov, c->cc64, z), count_launch();
    } else {
        gemv_kernel<float><<<egrid(c->n), 256, 0, s>>>(c->inv32, c->bc, c->n, c->cc32), count_launch();
        prolong_kernel<T, float><<<egrid(ov.nelem), 256, 0, s>>>(ov, c->cc32, z), count_launch();
    }
    RTG_CUDA(cudaGetLastError());
}

template void apply_coarse<double>(rtg_handle*, const double*, double*, cudaStream_t);
template void apply_coarse<float>(rtg_handle*, const float*, float*, cudaStream_t);

}  // namespace rtg

// Matrix-free application of the RT DG operator and the small vector kernels
// around it.  One CTA per spatial column: the column's DOFs are contiguous
// (cell-major, then i, j, a), the scattering block is dense over the column's
// angular nodes and diagonal in the spatial node (i, j), and the streaming
// terms stay inside one element, so a column is the natural unit of work.
#include <cstdio>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kApplyThreads = 256;

__device__ __forceinline__ int gofs(int n) { return (n - 1) * n * (2 * n - 1) / 6; }

template <typename T>
__device__ __forceinline__ T tabs(T v) { return v < T(0) ? -v : v; }

// y = Op(flags) x for the DOFs of one column.
// kParity: apply the reference's drop rules (|entry| <= 1e-14 in the (M - S)
// blocks, |entry| <= 1e-15 in the face terms, skip of cross-cell scattering
// where |wx wy sigma| <= 1e-14) so FP64 results match the assembled matrices.
template <typename T, typename TX, bool kParity>
__global__ void __launch_bounds__(kApplyThreads)
apply_kernel(OpView<T> v, uint32_t flags, const TX* __restrict__ x, TX* __restrict__ y) {
    const int ci = blockIdx.x;
    const ColDev C = v.cols[ci];
    const bool sys = flags & RTG_SYSTEM;
    const bool do_scat = sys || (flags & RTG_SCAT);
    const bool do_mass = sys || (flags & RTG_MASS);
    const bool merged = do_scat && do_mass;   // (M - S) block with the joint drop rule
    const bool do_ic = sys || (flags & RTG_IC);
    const T ic_sign = sys ? T(-1) : T(1);
    const bool do_bc = sys || (flags & RTG_BC);
    const bool mask_rows = flags & RTG_MASK_ROWS;
    const T small = T(kSmall), bctol = T(kBcTol);
    const T* W = v.W + v.W_off[C.sig];
    const T* wxs = v.lglw + C.nx * kMaxNodes;
    const T* wys = v.lglw + C.ny * kMaxNodes;
    const T* Gx = v.G + gofs(C.nx);
    const T* Gy = v.G + gofs(C.ny);
    const T dxdy8 = T(C.dx * C.dy / 8.);

    for (int e = C.elem_begin; e < C.elem_end; ++e) {
        const ElemDev E = v.elems[e];
        const int nth = E.nth;
        const int nloc = C.nx * C.ny * nth;
        const TX* xe = x + E.dof_off;
        const T* A = v.ang + E.ang;
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            const int r = l % nth;
            const int ij = l / nth;
            const int j = ij % C.ny;
            const int i = ij / C.ny;
            const int bm = E.flags >> 4;
            const bool bdry = ((bm & 1) && i == C.nx - 1) || ((bm & 2) && j == C.ny - 1) ||
                              ((bm & 4) && i == 0) || ((bm & 8) && j == 0);
            if (mask_rows && bdry) {
                y[E.dof_off + l] = TX(0);
                continue;
            }
            T acc = T(0);
            const int node = C.node_off + ij;
            // ---- extinction and scattering (rt/preconditioner_matrix.py:363-514)
            if (do_scat) {
                const T swv = v.sw[node];
                const T cw = dxdy8 * swv;
                const T* Wr = W + (int64_t)(E.row + r) * C.nth_col;
                const bool skip_cross = kParity && !(tabs(swv) > small);
                for (int e1 = C.elem_begin; e1 < C.elem_end; ++e1) {
                    if (skip_cross && e1 != e) continue;
                    const ElemDev E1 = v.elems[e1];
                    const TX* x1 = x + E1.dof_off + (int64_t)ij * E1.nth;
                    const T* W1 = Wr + E1.row;
                    for (int a = 0; a < E1.nth; ++a) {
                        T val = -cw * W1[a];
                        if (merged && e1 == e && a == r)
                            val += dxdy8 * T(E.dth) * A[r] * v.kw[node];
                        if (kParity && !(tabs(val) > small)) continue;
                        acc += val * T(x1[a]);
                    }
                }
            }
            if (do_mass && !merged) {
                acc += dxdy8 * T(E.dth) * A[r] * v.kw[node] * T(xe[l]);
            }
            // ---- interior streaming (rt/interior_convection_matrix.py:161-243)
            if (do_ic) {
                T t1 = T(0), t2 = T(0);
                const T* gy = Gy + j * C.ny;
                const TX* xi = xe + (int64_t)i * C.ny * nth + r;
                for (int jj = 0; jj < C.ny; ++jj) t1 += gy[jj] * T(xi[jj * nth]);
                const T* gx = Gx + i * C.nx;
                const TX* xj = xe + (int64_t)j * nth + r;
                for (int ii = 0; ii < C.nx; ++ii) t2 += gx[ii] * T(xj[(int64_t)ii * C.ny * nth]);
                const T ic = T(C.dx * E.dth / 4.) * wxs[i] * A[nth + r] * t1 +
                             T(C.dy * E.dth / 4.) * wys[j] * A[2 * nth + r] * t2;
                acc += ic_sign * ic;
            }
            // ---- face terms (rt/boundary_convection_matrix.py:258-524)
            if (do_bc) {
                for (int F = 0; F < 4; ++F) {
                    const bool on = (F == 0 && i == C.nx - 1) || (F == 1 && j == C.ny - 1) ||
                                    (F == 2 && i == 0) || (F == 3 && j == 0);
                    if (!on) continue;
                    if (E.flags & (1 << F)) {
                        const T dc = (F % 2 == 0) ? T(C.dy * E.dth / 4.) : T(C.dx * E.dth / 4.);
                        const T w = (F % 2 == 0) ? wys[j] : wxs[i];
                        const T val = dc * w * A[r] * A[(3 + F) * nth + r];
                        if (!kParity || tabs(val) > bctol) acc += val * T(xe[l]);
                        continue;
                    }
                    const int q = (F % 2 == 0) ? j : i;
                    const int n0 = (F % 2 == 0) ? C.ny : C.nx;
                    for (int k = E.cpl_begin; k < E.cpl_end; ++k) {
                        const CplDev cp = v.cpls[k];
                        if (cp.face != F) continue;
                        const ElemDev E1 = v.elems[cp.nbr];
                        const ColDev C1 = v.cols[E1.col];
                        const int nth1 = E1.nth;
                        const T* Es = v.mort + cp.es;
                        const T* Et = v.mort + cp.et;
                        const T dc = T(cp.dcoeff);
                        int64_t base, stride;
                        int m1;
                        if (F % 2 == 0) {
                            const int xi1 = (F == 0) ? 0 : C1.nx - 1;
                            base = E1.dof_off + (int64_t)xi1 * C1.ny * nth1;
                            stride = nth1;
                            m1 = C1.ny;
                        } else {
                            const int yi1 = (F == 1) ? 0 : C1.ny - 1;
                            base = E1.dof_off + (int64_t)yi1 * nth1;
                            stride = (int64_t)C1.ny * nth1;
                            m1 = C1.nx;
                        }
                        for (int jj = 0; jj < m1; ++jj) {
                            const T es = dc * Es[jj * n0 + q];
                            const TX* xl = x + base + jj * stride;
                            for (int a = 0; a < nth1; ++a) {
                                if (kParity) {
                                    const T val = T(cp.dcoeff) * Es[jj * n0 + q] * Et[a * nth + r];
                                    if (tabs(val) > bctol) acc += val * T(xl[a]);
                                } else {
                                    acc += es * Et[a * nth + r] * T(xl[a]);
                                }
                            }
                        }
                    }
                }
            }
            y[E.dof_off + l] = TX(acc);
        }
    }
}

__device__ __forceinline__ bool is_bdry(const ElemDev& E, const ColDev& C, int l) {
    const int bm = E.flags >> 4;
    if (!bm) return false;
    const int ij = l / E.nth;
    const int j = ij % C.ny;
    const int i = ij / C.ny;
    return ((bm & 1) && i == C.nx - 1) || ((bm & 2) && j == C.ny - 1) || ((bm & 4) && i == 0) ||
           ((bm & 8) && j == 0);
}

// One CTA per element for the elementwise kernels.
__global__ void interior_mask_kernel(OpView<double> v, uint8_t* mask) {
    const ElemDev E = v.elems[blockIdx.x];
    const ColDev C = v.cols[E.col];
    const int nloc = C.nx * C.ny * E.nth;
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) mask[E.dof_off + l] = is_bdry(E, C, l) ? 0 : 1;
}

__global__ void mask_vector_kernel(OpView<double> v, int part, const double* x, double* out) {
    const ElemDev E = v.elems[blockIdx.x];
    const ColDev C = v.cols[E.col];
    const int nloc = C.nx * C.ny * E.nth;
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
        const bool b = is_bdry(E, C, l);
        const bool keep = (part == 0) ? !b : b;
        out[E.dof_off + l] = keep ? x[E.dof_off + l] : 0.;
    }
}

// f_beta = (dx dy dth/8) wx_i wy_j wth_a f(x_i, y_j, th_a) (rt/forcing_vector.py:141-154)
__global__ void weight_forcing_kernel(OpView<double> v, const double* f, double* out) {
    const ElemDev E = v.elems[blockIdx.x];
    const ColDev C = v.cols[E.col];
    const int nloc = C.nx * C.ny * E.nth;
    const double dc = C.dx * C.dy * E.dth / 8.;
    const double* wx = v.lglw + C.nx * kMaxNodes;
    const double* wy = v.lglw + C.ny * kMaxNodes;
    const double* wt = v.ang + E.ang;
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
        const int r = l % E.nth;
        const int ij = l / E.nth;
        const int j = ij % C.ny;
        const int i = ij / C.ny;
        out[E.dof_off + l] = dc * wx[i] * wy[j] * wt[r] * f[E.dof_off + l];
    }
}

}  // namespace

template <typename T>
void launch_apply(const rtg_handle* h, const OpView<T>& v, uint32_t flags, const T* x, T* y,
                  cudaStream_t s) {
    if (sizeof(T) == 8)
        apply_kernel<T, T, true><<<v.ncols, kApplyThreads, 0, s>>>(v, flags, x, y);
    else
        apply_kernel<T, T, false><<<v.ncols, kApplyThreads, 0, s>>>(v, flags, x, y);
    RTG_CUDA(cudaGetLastError());
}

template void launch_apply<double>(const rtg_handle*, const OpView<double>&, uint32_t, const double*,
                                   double*, cudaStream_t);
template void launch_apply<float>(const rtg_handle*, const OpView<float>&, uint32_t, const float*,
                                  float*, cudaStream_t);

void launch_interior_mask(const rtg_handle* h, uint8_t* mask, cudaStream_t s) {
    interior_mask_kernel<<<h->v64.nelem, 128, 0, s>>>(h->v64, mask);
    RTG_CUDA(cudaGetLastError());
}

void launch_mask_vector(const rtg_handle* h, int part, const double* x, double* out, cudaStream_t s) {
    mask_vector_kernel<<<h->v64.nelem, 128, 0, s>>>(h->v64, part, x, out);
    RTG_CUDA(cudaGetLastError());
}

void launch_weight_forcing(const rtg_handle* h, const double* f, double* out, cudaStream_t s) {
    weight_forcing_kernel<<<h->v64.nelem, 128, 0, s>>>(h->v64, f, out);
    RTG_CUDA(cudaGetLastError());
}

}  // namespace rtg

// Matrix-free application of the RT DG operator and the small vector kernels
// around it.  One CTA per spatial column: the column's DOFs are contiguous
// (cell-major, then i, j, a), the scattering block is dense over the column's
// angular nodes and diagonal in the spatial node (i, j), and the streaming
// terms stay inside one element, so a column is the natural unit of work.
//
// Fast path (apply_col_kernel): the column's input is staged in shared memory
// transposed to [angular row R][spatial node ij] (and, when it fits, the
// column's angular scattering matrix W), then every output DOF is computed
// from shared memory and written in global order (coalesced).  Columns too
// large for shared memory use apply_global_kernel, which reads its operands
// from global memory.
#include <algorithm>
#include <cstdio>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kApplyThreads = 256;
constexpr int kMaxCellsStaged = 64;
constexpr size_t kSmemBudget = 200 * 1024;

__device__ __forceinline__ int gofs(int n) { return (n - 1) * n * (2 * n - 1) / 6; }

template <typename T>
__device__ __forceinline__ T tabs(T v) { return v < T(0) ? -v : v; }

__device__ __forceinline__ bool bdry_node(int bm, int i, int j, int nx, int ny) {
    return ((bm & 1) && i == nx - 1) || ((bm & 2) && j == ny - 1) || ((bm & 4) && i == 0) ||
           ((bm & 8) && j == 0);
}

// Face terms of one output node: outflow diagonal or inflow mortar couplings
// to neighbour elements (rt/boundary_convection_matrix.py:258-524).
// xself: the node's own input value.
template <typename T, typename TX, bool kParity>
__device__ __forceinline__ T face_terms(const OpView<T>& v, const float* __restrict__ mortf, const ColDev& C,
                                        const ElemDev& E, int e, int i, int j, int r, T xself,
                                        const TX* __restrict__ x) {
    const T bctol = T(kBcTol);
    const int nth = E.nth;
    const T* A = v.ang + E.ang;
    T acc = T(0);
    for (int F = 0; F < 4; ++F) {
        const bool on = (F == 0 && i == C.nx - 1) || (F == 1 && j == C.ny - 1) || (F == 2 && i == 0) ||
                        (F == 3 && j == 0);
        if (!on) continue;
        if (E.flags & (1 << F)) {
            const T dc = (F % 2 == 0) ? v.econst[4 * e + 2] : v.econst[4 * e + 1];
            const T w = (F % 2 == 0) ? v.lglw[C.ny * kMaxNodes + j] : v.lglw[C.nx * kMaxNodes + i];
            const T val = dc * w * A[r] * A[(3 + F) * nth + r];
            if (!kParity || tabs(val) > bctol) acc += val * xself;
            continue;
        }
        const int q = (F % 2 == 0) ? j : i;
        const int n0 = (F % 2 == 0) ? C.ny : C.nx;
        for (int k = E.cpl_begin; k < E.cpl_end; ++k) {
            const CplDev cp = v.cpls[k];
            if (cp.face != F) continue;
            const CplGeo g = v.cgeo[k];
            const int nth1 = g.nth1, m1 = g.m1;
            const int64_t base = g.base, stride = g.stride;
            const T* Es = v.mort + cp.es;
            const T* Et = v.mort + cp.et;
            const T dc = v.cplc[k];
            for (int jj = 0; jj < m1; ++jj) {
                const T es = Es[jj * n0 + q];
                const TX* xl = x + base + jj * stride;
                if (kParity) {
                    // keep dcoeff*Es*Et iff |.| > 1e-15, tested in FP32 with an
                    // FP64 fallback within 1e-6 of the threshold; one FMA per term
                    const T des = dc * es;
                    const float fdes = fabsf((float)des);
                    const float hi = 1.e-15f * (1.f + 1.e-6f), lo = 1.e-15f * (1.f - 1.e-6f);
                    T s = T(0);
                    for (int a = 0; a < nth1; ++a) {
                        const T et = Et[a * nth + r];
                        const float pf = fdes * fabsf(mortf[cp.et + a * nth + r]);
                        bool keep = pf > hi;
                        if (!keep && pf >= lo) keep = tabs(des * et) > bctol;
                        s = fma(keep ? et : T(0), T(xl[a]), s);
                    }
                    acc += des * s;
                } else {
                    T s = T(0);
                    for (int a = 0; a < nth1; ++a) s += Et[a * nth + r] * T(xl[a]);
                    acc += dc * es * s;
                }
            }
        }
    }
    return acc;
}

struct ApplyFlags {
    bool scat, mass, merged, ic, bc, mask_rows;
    float ic_sign;
};

__device__ __forceinline__ ApplyFlags decode(uint32_t flags) {
    ApplyFlags f;
    const bool sys = flags & RTG_SYSTEM;
    f.scat = sys || (flags & RTG_SCAT);
    f.mass = sys || (flags & RTG_MASS);
    f.merged = f.scat && f.mass;   // (M - S) block with the joint drop rule
    f.ic = sys || (flags & RTG_IC);
    f.ic_sign = sys ? -1.f : 1.f;
    f.bc = sys || (flags & RTG_BC);
    f.mask_rows = flags & RTG_MASK_ROWS;
    return f;
}

// ---------------------------------------------------------------- fast path
// Work item: outputs [begin, end) of one column (columns are split into
// chunks so that the heaviest columns do not serialise the launch).
// Shared memory: Xs[Nth][nij] | Ws[Nth][ldw] (optional) | Wf (FP32 copy of
// Ws, FP64 parity path only) | cell tables.
template <typename T, typename TX, bool kParity>
__global__ void __launch_bounds__(kApplyThreads)
apply_col_kernel(OpView<T> v, const float* __restrict__ Wf32, const float* __restrict__ mortf, uint32_t flags,
                 const int4* __restrict__ items,
                 int stage_w, const TX* __restrict__ x, TX* __restrict__ y) {
    extern __shared__ unsigned char smraw[];
    const int4 it = items[blockIdx.x];
    const int ci = it.x;
    const ColDev C = v.cols[ci];
    const ApplyFlags fl = decode(flags);
    const int nij = C.nx * C.ny, Nth = C.nth_col, ncell = C.elem_end - C.elem_begin;
    const int ldw = Nth | 1;   // odd row stride: rows of W land in different banks
    T* Xs = reinterpret_cast<T*>(smraw);
    T* Ws = Xs + (size_t)Nth * nij;
    float* Wf = reinterpret_cast<float*>(Ws + (stage_w ? (size_t)Nth * ldw : 0));
    const bool stage_f = kParity && stage_w;
    int* cbeg = reinterpret_cast<int*>(Wf + (stage_f ? (size_t)Nth * ldw : 0));  // [ncell+1] local DOF start
    int* crow = cbeg + ncell + 1;                                                  // [ncell] first row
    if (threadIdx.x == 0) {
        int off = 0;
        for (int k = 0; k < ncell; ++k) {
            const ElemDev E = v.elems[C.elem_begin + k];
            cbeg[k] = off;
            crow[k] = E.row;
            off += nij * E.nth;
        }
        cbeg[ncell] = off;
    }
    __syncthreads();
    const TX* xc = x + C.dof_off;
    // stage x transposed: Xs[(row_e + a) * nij + ij] = x[off_e + ij*nth + a]
    for (int d = threadIdx.x; d < C.ndof; d += blockDim.x) {
        int k = 0;
        while (d >= cbeg[k + 1]) ++k;
        const int nth = (cbeg[k + 1] - cbeg[k]) / nij;
        const int l = d - cbeg[k];
        Xs[(crow[k] + l % nth) * nij + l / nth] = T(xc[d]);
    }
    const T* Wg = v.W + v.W_off[C.sig];
    const float* Wgf = Wf32 + v.W_off[C.sig];
    if (stage_w)
        for (int t = threadIdx.x; t < Nth * Nth; t += blockDim.x) {
            const int row = t / Nth, col = t % Nth;
            Ws[row * ldw + col] = Wg[t];
            if (stage_f) Wf[row * ldw + col] = Wgf[t];
        }
    __syncthreads();
    const T small = T(kSmall);
    const T dxdy8 = v.colc[ci];
    const T* Gx = v.G + gofs(C.nx);
    const T* Gy = v.G + gofs(C.ny);
    TX* yc = y + C.dof_off;
    for (int d = it.y + threadIdx.x; d < it.z; d += blockDim.x) {
        int k = 0;
        while (d >= cbeg[k + 1]) ++k;
        const int e = C.elem_begin + k;
        const int nth = (cbeg[k + 1] - cbeg[k]) / nij;
        const int l = d - cbeg[k];
        const int r = l % nth, ij = l / nth, j = ij % C.ny, i = ij / C.ny;
        const ElemDev E = v.elems[e];
        const int bm = E.flags >> 4;
        if (fl.mask_rows && bdry_node(bm, i, j, C.nx, C.ny)) {
            yc[d] = TX(0);
            continue;
        }
        const int R = crow[k] + r;
        const T* A = v.ang + E.ang;
        const T xself = Xs[R * nij + ij];
        const int node = C.node_off + ij;
        T acc = T(0);
        if (fl.scat) {
            const T swv = v.sw[node];
            const T cw = dxdy8 * swv;
            const T mself = fl.merged ? v.econst[4 * e] * A[r] * v.kw[node] : T(0);
            if (kParity) {
                // Reference drop rules (rt/preconditioner_matrix.py:450-495):
                // keep -cw*W[R][c] iff |cw*W[R][c]| > 1e-14; cross-cell terms
                // only where |wx wy sigma| > 1e-14; the diagonal joins the
                // extinction term before its test.  The test runs in FP32 and
                // falls back to FP64 within 1e-6 (relative) of the threshold,
                // so the FP64 pipe does one FMA per term.
                const bool skip_cross = !(tabs(swv) > small);
                const int c0 = skip_cross ? crow[k] : 0;
                const int c1 = skip_cross ? crow[k] + nth : Nth;
                const float cwf = fabsf((float)cw);
                const float hi = 1.e-14f * (1.f + 1.e-6f), lo = 1.e-14f * (1.f - 1.e-6f);
                T s = T(0);
                for (int c = c0; c < c1; ++c) {
                    const T wv = stage_w ? Ws[R * ldw + c] : Wg[(int64_t)R * Nth + c];
                    const float wf = stage_f ? Wf[R * ldw + c] : Wgf[(int64_t)R * Nth + c];
                    const float pf = cwf * fabsf(wf);
                    bool keep = pf > hi;
                    if (!keep && pf >= lo) keep = tabs(cw * wv) > small;
                    s = fma(keep && c != R ? wv : T(0), Xs[c * nij + ij], s);
                }
                const T wd = stage_w ? Ws[R * ldw + R] : Wg[(int64_t)R * Nth + R];
                const T vd = mself - cw * wd;
                acc = -cw * s + (tabs(vd) > small ? vd : T(0)) * xself;
            } else {
                T s = T(0);
                if (stage_w) {
                    const T* wr = Ws + R * ldw;
#pragma unroll 4
                    for (int c = 0; c < Nth; ++c) s += wr[c] * Xs[c * nij + ij];
                } else {
                    const T* wr = Wg + (int64_t)R * Nth;
#pragma unroll 4
                    for (int c = 0; c < Nth; ++c) s += wr[c] * Xs[c * nij + ij];
                }
                acc = -cw * s + mself * xself;
            }
        }
        if (fl.mass && !fl.merged) acc += v.econst[4 * e] * A[r] * v.kw[node] * xself;
        if (fl.ic) {
            // interior streaming, sum-factorised (rt/interior_convection_matrix.py:161-243)
            const T* xr = Xs + R * nij;
            T t1 = T(0), t2 = T(0);
            const T* gy = Gy + j * C.ny;
            for (int jj = 0; jj < C.ny; ++jj) t1 += gy[jj] * xr[i * C.ny + jj];
            const T* gx = Gx + i * C.nx;
            for (int ii = 0; ii < C.nx; ++ii) t2 += gx[ii] * xr[ii * C.ny + j];
            const T ic = v.econst[4 * e + 1] * v.lglw[C.nx * kMaxNodes + i] * A[nth + r] * t1 +
                         v.econst[4 * e + 2] * v.lglw[C.ny * kMaxNodes + j] * A[2 * nth + r] * t2;
            acc += T(fl.ic_sign) * ic;
        }
        if (fl.bc && (i == 0 || j == 0 || i == C.nx - 1 || j == C.ny - 1))
            acc += face_terms<T, TX, kParity>(v, mortf, C, E, e, i, j, r, xself, x);
        yc[d] = TX(acc);
    }
}

// ------------------------------------------------------------ global path
template <typename T, typename TX, bool kParity>
__global__ void __launch_bounds__(kApplyThreads)
apply_global_kernel(OpView<T> v, const float* __restrict__ mortf, uint32_t flags, const int32_t* __restrict__ cols,
                    const TX* __restrict__ x, TX* __restrict__ y) {
    const int ci = cols[blockIdx.x];
    const ColDev C = v.cols[ci];
    const ApplyFlags fl = decode(flags);
    const T small = T(kSmall);
    const T* W = v.W + v.W_off[C.sig];
    const T* Gx = v.G + gofs(C.nx);
    const T* Gy = v.G + gofs(C.ny);
    const T dxdy8 = v.colc[ci];
    for (int e = C.elem_begin; e < C.elem_end; ++e) {
        const ElemDev E = v.elems[e];
        const int nth = E.nth;
        const int nloc = C.nx * C.ny * nth;
        const TX* xe = x + E.dof_off;
        const T* A = v.ang + E.ang;
        for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
            const int r = l % nth, ij = l / nth, j = ij % C.ny, i = ij / C.ny;
            if (fl.mask_rows && bdry_node(E.flags >> 4, i, j, C.nx, C.ny)) {
                y[E.dof_off + l] = TX(0);
                continue;
            }
            T acc = T(0);
            const int node = C.node_off + ij;
            const T xself = T(xe[l]);
            if (fl.scat) {
                const T swv = v.sw[node];
                const T cw = dxdy8 * swv;
                const T* Wr = W + (int64_t)(E.row + r) * C.nth_col;
                const bool skip_cross = kParity && !(tabs(swv) > small);
                const T mself = fl.merged ? v.econst[4 * e] * A[r] * v.kw[node] : T(0);
                for (int e1 = C.elem_begin; e1 < C.elem_end; ++e1) {
                    if (skip_cross && e1 != e) continue;
                    const ElemDev E1 = v.elems[e1];
                    const TX* x1 = x + E1.dof_off + (int64_t)ij * E1.nth;
                    const T* W1 = Wr + E1.row;
                    for (int a = 0; a < E1.nth; ++a) {
                        T val = -cw * W1[a];
                        if (e1 == e && a == r) val += mself;
                        if (kParity && !(tabs(val) > small)) continue;
                        acc += val * T(x1[a]);
                    }
                }
            }
            if (fl.mass && !fl.merged) acc += v.econst[4 * e] * A[r] * v.kw[node] * xself;
            if (fl.ic) {
                T t1 = T(0), t2 = T(0);
                const T* gy = Gy + j * C.ny;
                const TX* xi = xe + (int64_t)i * C.ny * nth + r;
                for (int jj = 0; jj < C.ny; ++jj) t1 += gy[jj] * T(xi[jj * nth]);
                const T* gx = Gx + i * C.nx;
                const TX* xj = xe + (int64_t)j * nth + r;
                for (int ii = 0; ii < C.nx; ++ii) t2 += gx[ii] * T(xj[(int64_t)ii * C.ny * nth]);
                const T ic = v.econst[4 * e + 1] * v.lglw[C.nx * kMaxNodes + i] * A[nth + r] * t1 +
                             v.econst[4 * e + 2] * v.lglw[C.ny * kMaxNodes + j] * A[2 * nth + r] * t2;
                acc += T(fl.ic_sign) * ic;
            }
            if (fl.bc && (i == 0 || j == 0 || i == C.nx - 1 || j == C.ny - 1))
                acc += face_terms<T, TX, kParity>(v, mortf, C, E, e, i, j, r, xself, x);
            y[E.dof_off + l] = TX(acc);
        }
    }
}

__device__ __forceinline__ bool is_bdry(const ElemDev& E, const ColDev& C, int l) {
    const int bm = E.flags >> 4;
    if (!bm) return false;
    const int ij = l / E.nth;
    return bdry_node(bm, ij / C.ny, ij % C.ny, C.nx, C.ny);
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

// Work partition of the fast path, per precision: columns whose staged input
// stays within the shared-memory budget, cut into chunks of at most kChunk
// outputs, heaviest chunks first, in two launch groups: with the column's W
// staged too, or (large angular meshes) with W read through L2.
constexpr int kChunk = 1024;

struct ApplyGroup {
    int4* d_items = nullptr;
    int nitems = 0;
    size_t smem = 0;
    int stage_w = 0;
};

struct ApplyPlan {
    ApplyGroup g[2];            // 0: input and W staged; 1: input staged, W read through L2
    int32_t* d_slow = nullptr;
    int nslow = 0;
    std::vector<void*> allocs;
};

template <typename T>
static ApplyPlan* make_plan(const rtg_handle* h) {
    const HostTables& t = h->host;
    constexpr bool parity = sizeof(T) == 8;
    ApplyPlan* p = new ApplyPlan();
    std::vector<std::pair<int64_t, int4>> items[2];
    std::vector<int32_t> slow;
    size_t need[2] = {0, 0};
    for (int ci = 0; ci < (int)t.cols.size(); ++ci) {
        const ColDev& C = t.cols[ci];
        const int ncell = C.elem_end - C.elem_begin;
        const size_t sx = sizeof(T) * (size_t)C.ndof + sizeof(int) * (2 * ncell + 2) + 16;
        const size_t sw = (sizeof(T) + (parity ? sizeof(float) : 0)) * (size_t)C.nth_col * (C.nth_col | 1);
        if (sx > kSmemBudget || ncell > kMaxCellsStaged) {
            slow.push_back(ci);
            continue;
        }
        const int grp = (sx + sw <= kSmemBudget) ? 0 : 1;
        need[grp] = std::max(need[grp], grp == 0 ? sx + sw : sx);
        const int nch = (C.ndof + kChunk - 1) / kChunk;
        const int per = (C.ndof + nch - 1) / nch;
        for (int q = 0; q < nch; ++q) {
            const int b0 = q * per, b1 = std::min(C.ndof, b0 + per);
            items[grp].push_back({(int64_t)(b1 - b0) * (C.nth_col + C.nx + C.ny) + C.ndof, make_int4(ci, b0, b1, 0)});
        }
    }
    auto up = [&](const void* src, size_t bytes) -> void* {
        void* d = nullptr;
        RTG_CUDA(cudaMalloc(&d, std::max<size_t>(bytes, 16)));
        p->allocs.push_back(d);
        if (bytes) RTG_CUDA(cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice));
        return d;
    };
    for (int grp = 0; grp < 2; ++grp) {
        std::stable_sort(items[grp].begin(), items[grp].end(), [](auto& a, auto& b) { return a.first > b.first; });
        std::vector<int4> it4;
        for (auto& pr : items[grp]) it4.push_back(pr.second);
        ApplyGroup& G = p->g[grp];
        G.nitems = (int)it4.size();
        G.stage_w = grp == 0 ? 1 : 0;
        G.smem = need[grp];
        G.d_items = (int4*)up(it4.data(), sizeof(int4) * it4.size());
    }
    p->nslow = (int)slow.size();
    p->d_slow = (int32_t*)up(slow.data(), sizeof(int32_t) * slow.size());
    return p;
}

void free_apply_plans(rtg_handle* h) {
    for (ApplyPlan* p : {h->plan64, h->plan32}) {
        if (!p) continue;
        for (void* d : p->allocs) cudaFree(d);
        delete p;
    }
    h->plan64 = h->plan32 = nullptr;
}

template <typename T>
void launch_apply(const rtg_handle* hc, const OpView<T>& v, uint32_t flags, const T* x, T* y,
                  cudaStream_t s) {
    rtg_handle* h = const_cast<rtg_handle*>(hc);
    constexpr bool f64 = sizeof(T) == 8;
    ApplyPlan*& plan = f64 ? h->plan64 : h->plan32;
    if (!plan) {
        plan = make_plan<T>(h);
        size_t mx = std::max(plan->g[0].smem, plan->g[1].smem);
        if (mx > 48 * 1024)
            RTG_CUDA(cudaFuncSetAttribute(apply_col_kernel<T, T, f64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)mx));
    }
    for (int grp = 0; grp < 2; ++grp) {
        const ApplyGroup& G = plan->g[grp];
        if (G.nitems)
            apply_col_kernel<T, T, f64><<<G.nitems, kApplyThreads, G.smem, s>>>(v, h->v32.W, h->v32.mort, flags,
                                                                              G.d_items, G.stage_w, x, y);
    }
    if (plan->nslow)
        apply_global_kernel<T, T, f64><<<plan->nslow, kApplyThreads, 0, s>>>(v, h->v32.mort, flags, plan->d_slow, x, y);
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

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
#include <map>
#include <string>
#include <tuple>

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
    if (v.stop && *v.stop) return;
    const int4 it = items[blockIdx.x];
    const int ci = it.x;
    if (v.skip && v.skip[ci]) return;
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
    // (d grows per thread, so the cell index k only moves forward)
    int k = 0;
    for (int d = threadIdx.x; d < C.ndof; d += blockDim.x) {
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
    k = 0;
    for (int d = it.y + threadIdx.x; d < it.z; d += blockDim.x) {
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

// ------------------------------------------------------------ tiled path
// Work item: whole cells [cell_begin, cell_end) of one column, i.e. the
// rectangle of angular rows R0 .. R0+M-1 times all nij spatial nodes.  The
// scattering of the item is the product Y[m][ij] = sum_c W[R0+m][c] X[c][ij]
// over all Nth angular nodes of the column; it runs from shared memory with
// 4 x 4 register tiles (16 FMAs per eight loaded values).  The epilogue adds
// extinction, streaming and face terms and writes y in global order.
// The inflow face fluxes of the item's elements are factorised per coupling
// (T[jj][r] = sum_a Et[a][r] x_nbr[jj][a], then sum_jj Es[jj][q] T[jj][r]) and
// accumulated into Fy before the epilogue; T and Fy reuse the W region.
// Shared memory: Xs[Nth][nijp] | WsT[Nth][Mp] (later T | Fy[Mp][nijp]) |
// Ys[Mp][nijp] | cell tables.
//
// FP64 (kParity) keeps the reference's drop rules without per-term tests on
// the common path:
//  * scattering: W's diagonal is left out of the product, and each spatial
//    node has a class computed on the host with the exact FP64 test: every
//    nonzero off-diagonal term kept (use Y), none kept (0), or mixed (the
//    per-term loop with the FP32-prefiltered test); the diagonal joins the
//    extinction term before its test (rt/preconditioner_matrix.py:450-495);
//  * faces: a coupling whose dropped terms (|dcoeff Es Et| <= 1e-15) are
//    exactly the products with a set of Es entries or a set of Et entries
//    (round-off-sized mortar entries) uses cleaned copies of dcoeff*Es and
//    Et with those entries zeroed, so the factorised flux sums exactly the
//    kept terms; any other coupling is summed term by term with the test
//    (rt/boundary_convection_matrix.py:258-524).
struct TileItem {
    int col, cell_begin, cell_end, row0;
    int cpl_begin, cpl_end;   // entries of the item's couplings
    int tsz;                  // values of T (padded to 4)
    int wcap;                 // values of the W region
    int ttot, ctot;           // work items of the two flux phases (ctot: boundary nodes x rows)
};

// One coupling of a tiled item: where its neighbour line is, its mortars,
// and its offsets in the two flux phases.  FP64: es and et index the cleaned
// tables (dcoeff*Es and Et); k is the coupling, tested marks a coupling summed
// term by term.
struct TileCpl {
    int64_t base;             // neighbour line: x[base + jj*stride + a]
    int rowloc, nth, toff, coff;
    int m1, nt1, n0, face;
    int stride, es, et;
    float dc;
    int k, tested;
};
constexpr int kMaxItemCpl = 96;
constexpr int kMaxItemCells = 128;

// Host-built tables of the FP64 tiled path.
template <typename T>
struct TileParity {
    const uint8_t* scls = nullptr;   // per spatial node: 0 no, 1 every, 2 some off-diagonal scattering term kept
    const T* mortc = nullptr;        // cleaned dcoeff*Es and Et per coupling
    const float* mortf = nullptr;    // FP32 copy of the mortars (tested couplings)
    const float* Wf = nullptr;       // FP32 copy of W (mixed nodes without a mask)
    const uint64_t* colfull = nullptr;   // per column: bit ij set when node ij is of class 1 (ij < 64)
    const int64_t* kbase = nullptr;      // per spatial node of class 2: first keep mask, or -1
    const uint64_t* kmask = nullptr;     // per (class-2 node, row R): bit c set when term (R, c) is kept
};

// f-th node on the boundary of an nx x ny node grid, going around (j = 0 row,
// i = nx-1 column, j = ny-1 row, i = 0 column), each node once
__device__ __forceinline__ void boundary_node(int f, int nx, int ny, int& i, int& j) {
    if (nx == 1 || ny == 1) {   // a single row or column: every node is on the boundary
        i = nx == 1 ? 0 : f;
        j = nx == 1 ? f : 0;
        return;
    }
    if (f < nx) { i = f; j = 0; return; }
    f -= nx;
    if (f < ny - 1) { i = nx - 1; j = f + 1; return; }
    f -= ny - 1;
    if (f < nx - 1) { i = nx - 2 - f; j = ny - 1; return; }
    f -= nx - 1;
    i = 0;
    j = ny - 2 - f;
}

__host__ __device__ __forceinline__ int boundary_nodes(int nx, int ny) {
    return (nx == 1 || ny == 1) ? nx * ny : 2 * (nx + ny) - 4;
}

// four consecutive values from 16-byte-aligned shared memory
__device__ __forceinline__ void load4(const float* p, float o[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
}
__device__ __forceinline__ void load4(const double* p, double o[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    const double2 b = *reinterpret_cast<const double2*>(p + 2);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
}
__device__ __forceinline__ void store4(float* p, const float v[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void store4(double* p, const double v[4]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

template <typename T, bool kParity>
__global__ void __launch_bounds__(kApplyThreads)
apply_tiled_kernel(OpView<T> v, TileParity<T> par, uint32_t flags, const TileItem* __restrict__ items,
                   const TileCpl* __restrict__ cpl_ent, const T* __restrict__ x, T* __restrict__ y) {
    extern __shared__ double2 smt4[];
    __shared__ TileCpl sc[kMaxItemCpl];
    __shared__ int4 s_el[kMaxItemCells];      // per item cell: first entry, end entry, local row, nth
    __shared__ int s_po[kMaxItemCells + 1];   // prefix of boundary nodes x nth
    T* smt = reinterpret_cast<T*>(smt4);
    if (v.stop && *v.stop) return;
    const TileItem it = items[blockIdx.x];
    const int ci = it.col;
    if (v.skip && v.skip[ci]) return;
    const ColDev C = v.cols[ci];
    const ApplyFlags fl = decode(flags);
    const int nij = C.nx * C.ny, Nth = C.nth_col, ncell = C.elem_end - C.elem_begin;
    const int nijp = (nij + 3) & ~3;
    const int M = [&] {
        int m = 0;
        for (int k = it.cell_begin; k < it.cell_end; ++k) m += v.elems[C.elem_begin + k].nth;
        return m;
    }();
    const int Mp = (M + 3) & ~3;
    T* Xs = smt;                                  // [Nth][nijp]
    T* WsT = Xs + (size_t)Nth * nijp;             // [Nth][Mp]
    T* Ys = WsT + (size_t)it.wcap;                // [Mp][nijp]
    T* Tb = WsT;                                  // after the product: T
    T* Fy = WsT + it.tsz;                         //                    Fy[Mp][nijp]
    int* cbeg = reinterpret_cast<int*>(Ys + (size_t)Mp * nijp);   // [ncell+1] local DOF start
    int* crow = cbeg + ncell + 1;                                  // [ncell] first row
    if (threadIdx.x == 0) {
        int off = 0;
        for (int k = 0; k < ncell; ++k) {
            const ElemDev E = v.elems[C.elem_begin + k];
            cbeg[k] = off;
            crow[k] = E.row;
            off += nij * E.nth;
        }
        cbeg[ncell] = off;
        int eb = 0, po = 0;
        for (int k = it.cell_begin; k < it.cell_end; ++k) {
            const ElemDev E = v.elems[C.elem_begin + k];
            const int nc = E.cpl_end - E.cpl_begin;
            s_el[k - it.cell_begin] = make_int4(eb, eb + nc, E.row - it.row0, E.nth);
            s_po[k - it.cell_begin] = po;
            eb += nc;
            po += boundary_nodes(C.nx, C.ny) * E.nth;
        }
        s_po[it.cell_end - it.cell_begin] = po;
    }
    const int nent = it.cpl_end - it.cpl_begin;
    for (int q = threadIdx.x; q < nent; q += blockDim.x) sc[q] = cpl_ent[it.cpl_begin + q];
    __syncthreads();
    const T* xc = x + C.dof_off;
    // stage x transposed: Xs[row][ij]; pad columns are zero (d grows per
    // thread, so the cell index k only moves forward)
    {
        int k = 0;
        for (int d = threadIdx.x; d < C.ndof; d += blockDim.x) {
            while (d >= cbeg[k + 1]) ++k;
            const int nth = (cbeg[k + 1] - cbeg[k]) / nij;
            const int l = d - cbeg[k];
            Xs[(crow[k] + l % nth) * nijp + l / nth] = xc[d];
        }
    }
    if (nijp != nij)
        for (int t = threadIdx.x; t < Nth * (nijp - nij); t += blockDim.x)
            Xs[(t / (nijp - nij)) * nijp + nij + t % (nijp - nij)] = T(0);
    const T* Wg = v.W + v.W_off[C.sig];
    if (fl.scat) {
        for (int t = threadIdx.x; t < Nth * Mp; t += blockDim.x) {
            const int c = t / Mp, m = t % Mp;
            // FP64: the diagonal joins the extinction term in the epilogue
            const bool use = m < M && !(kParity && c == it.row0 + m);
            WsT[t] = use ? __ldg(Wg + (int64_t)(it.row0 + m) * Nth + c) : T(0);
        }
    }
    __syncthreads();
    if (fl.scat) {
        const int tm = Mp / 4, tn = nijp / 4;
        // FP64: only nodes of class 1 read the product
        const uint64_t fullm = kParity ? (nij <= 64 ? par.colfull[ci] : ~0ull) : ~0ull;
        for (int tile = threadIdx.x; tile < tm * tn; tile += blockDim.x) {
            const int m0 = 4 * (tile / tn), j0 = 4 * (tile % tn);
            if (kParity && j0 < 64 && !((fullm >> j0) & 0xFull)) continue;
            T acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll 4
            for (int c = 0; c < Nth; ++c) {
                T wv[4], xa[4];
                load4(WsT + c * Mp + m0, wv);
                load4(Xs + c * nijp + j0, xa);
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(wv[i], xa[j], acc[i][j]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) store4(Ys + (m0 + i) * nijp + j0, acc[i]);
        }
    }
    __syncthreads();
    // inflow face fluxes of the item's elements into Fy (the W region is free)
    if (fl.bc) {
        for (int t = threadIdx.x; t < Mp * nijp; t += blockDim.x) Fy[t] = T(0);
        // T[jj][r] of every coupling, flattened over (coupling, jj, r); t
        // grows per thread, so the coupling index only moves forward
        {
            int c = 0;
            for (int t = threadIdx.x; t < it.ttot; t += blockDim.x) {
                while (t >= sc[c].toff + sc[c].m1 * sc[c].nth) ++c;
                const TileCpl& en = sc[c];
                if (kParity && en.tested) continue;   // summed term by term below
                const int q = t - en.toff, jj = q / en.nth, r = q % en.nth;
                const T* Et = (kParity ? par.mortc : v.mort) + en.et;
                const T* xl = x + en.base + (int64_t)jj * en.stride;
                T acc = T(0);
                for (int a = 0; a < en.nt1; ++a) acc = fma(Et[a * en.nth + r], xl[a], acc);
                Tb[t] = acc;
            }
        }
        __syncthreads();
        // one thread per (boundary node, row): the element's couplings on the
        // node's faces in a fixed order, so the sum is deterministic
        {
            int k = 0;
            for (int t = threadIdx.x; t < it.ctot; t += blockDim.x) {
                while (t >= s_po[k + 1]) ++k;
                const int4 el = s_el[k];
                const int f = (t - s_po[k]) / el.w, r = (t - s_po[k]) % el.w;
                int i, j;
                boundary_node(f, C.nx, C.ny, i, j);
                T acc = T(0);
                for (int c = el.x; c < el.y; ++c) {
                    const TileCpl& en = sc[c];
                    const int F = en.face;
                    const bool on = (F == 0 && i == C.nx - 1) || (F == 1 && j == C.ny - 1) || (F == 2 && i == 0) ||
                                    (F == 3 && j == 0);
                    if (!on) continue;
                    const int q = (F % 2 == 0) ? j : i;
                    if constexpr (kParity) {
                        if (en.tested) {
                            // keep dcoeff*Es*Et iff |.| > 1e-15, tested in FP32 with
                            // an FP64 fallback within 1e-6 of the threshold
                            const CplDev cp = v.cpls[en.k];
                            const T* Es = v.mort + cp.es;
                            const T* Et = v.mort + cp.et;
                            const T dc = v.cplc[en.k];
                            const float hi = 1.e-15f * (1.f + 1.e-6f), lo = 1.e-15f * (1.f - 1.e-6f);
                            for (int jj = 0; jj < en.m1; ++jj) {
                                const T des = dc * Es[jj * en.n0 + q];
                                const float fdes = fabsf((float)des);
                                const T* xl = x + en.base + (int64_t)jj * en.stride;
                                T s = T(0);
                                for (int a = 0; a < en.nt1; ++a) {
                                    const T et = Et[a * en.nth + r];
                                    const float pf = fdes * fabsf(par.mortf[cp.et + a * en.nth + r]);
                                    bool keep = pf > hi;
                                    if (!keep && pf >= lo) keep = tabs(des * et) > T(kBcTol);
                                    s = fma(keep ? et : T(0), xl[a], s);
                                }
                                acc += des * s;
                            }
                        } else {
                            const T* Es = par.mortc + en.es;
                            T sacc = T(0);
                            for (int jj = 0; jj < en.m1; ++jj)
                                sacc = fma(Es[jj * en.n0 + q], Tb[en.toff + jj * en.nth + r], sacc);
                            acc += sacc;
                        }
                    } else {
                        const T* Es = v.mort + en.es;
                        T sacc = T(0);
                        for (int jj = 0; jj < en.m1; ++jj)
                            sacc = fma(Es[jj * en.n0 + q], Tb[en.toff + jj * en.nth + r], sacc);
                        acc = fma(T(en.dc), sacc, acc);
                    }
                }
                Fy[(el.z + r) * nijp + i * C.ny + j] = acc;
            }
        }
        __syncthreads();
    }
    const T small = T(kSmall);
    const T dxdy8 = v.colc[ci];
    const T* Gx = v.G + gofs(C.nx);
    const T* Gy = v.G + gofs(C.ny);
    T* yc = y + C.dof_off;
    const int d0 = cbeg[it.cell_begin], d1 = cbeg[it.cell_end];
    int k = it.cell_begin;
    for (int d = d0 + threadIdx.x; d < d1; d += blockDim.x) {
        while (d >= cbeg[k + 1]) ++k;
        const int e = C.elem_begin + k;
        const int nth = (cbeg[k + 1] - cbeg[k]) / nij;
        const int l = d - cbeg[k];
        const int r = l % nth, ij = l / nth, j = ij % C.ny, i = ij / C.ny;
        const ElemDev E = v.elems[e];
        if (fl.mask_rows && bdry_node(E.flags >> 4, i, j, C.nx, C.ny)) {
            yc[d] = T(0);
            continue;
        }
        const int R = crow[k] + r;
        const T* A = v.ang + E.ang;
        const T xself = Xs[R * nijp + ij];
        const int node = C.node_off + ij;
        const T mterm = v.econst[4 * e] * A[r] * v.kw[node];
        T acc = T(0);
        if constexpr (kParity) {
            if (fl.scat) {
                const T swv = v.sw[node];
                const T cw = dxdy8 * swv;
                const int cls = par.scls[node];
                T s = T(0);
                if (cls == 1) {
                    s = Ys[(R - it.row0) * nijp + ij];
                } else if (cls == 2 && par.kbase[node] >= 0) {
                    // some terms kept, some dropped: the host's keep mask of row R
                    uint64_t mk = par.kmask[par.kbase[node] + R];
                    const T* wr = Wg + (int64_t)R * Nth;
                    while (mk) {
                        const int c = __ffsll((long long)mk) - 1;
                        mk &= mk - 1;
                        s = fma(wr[c], Xs[c * nijp + ij], s);
                    }
                } else if (cls == 2) {
                    // some terms kept, some dropped: test each one
                    const bool skip_cross = !(tabs(swv) > small);
                    const int c0 = skip_cross ? crow[k] : 0;
                    const int c1 = skip_cross ? crow[k] + nth : Nth;
                    const float cwf = fabsf((float)cw);
                    const float hi = 1.e-14f * (1.f + 1.e-6f), lo = 1.e-14f * (1.f - 1.e-6f);
                    const float* Wf = par.Wf + v.W_off[C.sig];
                    for (int c = c0; c < c1; ++c) {
                        const T wv = Wg[(int64_t)R * Nth + c];
                        const float pf = cwf * fabsf(Wf[(int64_t)R * Nth + c]);
                        bool keep = pf > hi;
                        if (!keep && pf >= lo) keep = tabs(cw * wv) > small;
                        s = fma(keep && c != R ? wv : T(0), Xs[c * nijp + ij], s);
                    }
                }
                const T vd = (fl.merged ? mterm : T(0)) - cw * Wg[(int64_t)R * Nth + R];
                acc = -cw * s + (tabs(vd) > small ? vd : T(0)) * xself;
            }
            if (fl.mass && !fl.merged) acc += mterm * xself;
        } else {
            if (fl.scat) acc = -dxdy8 * v.sw[node] * Ys[(R - it.row0) * nijp + ij];
            if (fl.mass) acc += mterm * xself;
        }
        if (fl.ic) {
            const T* xr = Xs + R * nijp;
            T t1 = T(0), t2 = T(0);
            const T* gy = Gy + j * C.ny;
            for (int jj = 0; jj < C.ny; ++jj) t1 += gy[jj] * xr[i * C.ny + jj];
            const T* gx = Gx + i * C.nx;
            for (int ii = 0; ii < C.nx; ++ii) t2 += gx[ii] * xr[ii * C.ny + j];
            const T ic = v.econst[4 * e + 1] * v.lglw[C.nx * kMaxNodes + i] * A[nth + r] * t1 +
                         v.econst[4 * e + 2] * v.lglw[C.ny * kMaxNodes + j] * A[2 * nth + r] * t2;
            acc += T(fl.ic_sign) * ic;
        }
        if (fl.bc && (i == 0 || j == 0 || i == C.nx - 1 || j == C.ny - 1)) {
            acc += Fy[(R - it.row0) * nijp + ij];
            // outflow faces: the diagonal term (rt/boundary_convection_matrix.py:276-346)
            for (int F = 0; F < 4; ++F) {
                if (!(E.flags & (1 << F))) continue;
                const bool on = (F == 0 && i == C.nx - 1) || (F == 1 && j == C.ny - 1) || (F == 2 && i == 0) ||
                                (F == 3 && j == 0);
                if (!on) continue;
                const T dc = (F % 2 == 0) ? v.econst[4 * e + 2] : v.econst[4 * e + 1];
                const T w = (F % 2 == 0) ? v.lglw[C.ny * kMaxNodes + j] : v.lglw[C.nx * kMaxNodes + i];
                const T val = dc * w * A[r] * A[(3 + F) * nth + r];
                if (!kParity || tabs(val) > T(kBcTol)) acc += val * xself;
            }
        }
        yc[d] = acc;
    }
}

// ------------------------------------------------------------ global path
template <typename T, typename TX, bool kParity>
__global__ void __launch_bounds__(kApplyThreads)
apply_global_kernel(OpView<T> v, const float* __restrict__ mortf, uint32_t flags, const int32_t* __restrict__ cols,
                    const TX* __restrict__ x, TX* __restrict__ y) {
    if (v.stop && *v.stop) return;
    const int ci = cols[blockIdx.x];
    if (v.skip && v.skip[ci]) return;
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
// The FP64 apply is FP64-pipe bound and, with large items, all of them fit in
// one wave, so the heaviest item sets the kernel time: smaller items balance
// the SMs (the item size is tuned per handle, tune_plan64).
constexpr int kChunk64 = 256;

struct ApplyGroup {
    int4* d_items = nullptr;
    int nitems = 0;
    size_t smem = 0;
    int stage_w = 0;
};

constexpr int kTileRows = 64;       // default row cap (before tuning)
constexpr int kTileOut = 2048;
constexpr int kTuneCaps[] = {16, 32, 64, 128};
constexpr int kNumTuneCaps = 4;

// Tuning record of one degree class: nx, ny, the column's angular nodes
// rounded up to a power of two, the chosen row cap, and the measured time (ns)
// of the class's items with each candidate cap (-1: not run).
struct TuneRecord {
    int nx, ny, nthb, cap;
    int ns[kNumTuneCaps];
};

// Tables of the FP64 tiled path (drop rules resolved on the host): the
// scattering class of every spatial node and the cleaned mortar products of
// every coupling.
struct ParityTables {
    uint8_t* d_scls = nullptr;
    double* d_mortc = nullptr;
    uint64_t* d_colfull = nullptr;
    int64_t* d_kbase = nullptr;
    uint64_t* d_kmask = nullptr;
    std::vector<int> esc, etc;     // per coupling: offsets of dcoeff*Es and Et in the cleaned table
    std::vector<char> tested;      // per coupling: summed term by term
    int64_t nodes[3] = {0, 0, 0};  // nodes per scattering class
    int64_t ntested = 0;
};

struct ApplyPlan {
    ApplyGroup g[2];            // 0: input and W staged; 1: input staged, W read through L2
    int32_t* d_slow = nullptr;
    int nslow = 0;
    TileItem* d_tiles = nullptr;   // tiled items
    TileCpl* d_tile_cpl = nullptr; // their coupling entries
    int ntiles = 0;
    size_t tile_smem = 0;
    const ParityTables* par = nullptr;   // FP64 tiled path
    bool own_par = false;
    std::vector<TuneRecord> tuning;
    std::vector<void*> allocs;
};

static void free_parity(const ParityTables* pt) {
    if (!pt) return;
    cudaFree(pt->d_scls);
    cudaFree(pt->d_mortc);
    cudaFree(pt->d_colfull);
    cudaFree(pt->d_kbase);
    cudaFree(pt->d_kmask);
    delete pt;
}

// Resolves the FP64 drop rules of the tiled path on the host, with the same
// FP64 products and comparisons the per-term path makes.
//  * node class: |fl(cw w)| grows with |w|, so the smallest and largest
//    nonzero off-diagonal |W| entries decide whether every, no or some
//    scattering term of the node is kept (cross-cell terms only where
//    |wx wy sigma| > 1e-14, rt/preconditioner_matrix.py:450-495);
//  * coupling: the terms dropped by |dcoeff Es Et| <= 1e-15 must be exactly
//    the products with a set of Es entries or a set of Et entries; then those
//    entries are zeroed in copies of dcoeff*Es and Et
//    (rt/boundary_convection_matrix.py:258-524).
static ParityTables* build_parity(const rtg_handle* h) {
    const HostTables& t = h->host;
    ParityTables* pt = new ParityTables();
    std::vector<uint8_t> scls((size_t)std::max(t.nnodes, 1), 0);
    std::vector<uint64_t> colfull(t.cols.size(), 0), kmask;
    std::vector<int64_t> kbase((size_t)std::max(t.nnodes, 1), -1);
    for (int ci = 0; ci < (int)t.cols.size(); ++ci) {
        const ColDev& C = t.cols[ci];
        const int Nth = C.nth_col, ncell = C.elem_end - C.elem_begin;
        const double* W = t.W.data() + t.W_off[C.sig];
        double wmin = 0., wmax = 0.;   // nonzero off-diagonal |W|, whole column
        std::vector<double> cmax(ncell, 0.);   // largest own-cell off-diagonal |W| per cell
        std::vector<int> rcell(Nth, 0);
        for (int k = 0; k < ncell; ++k) {
            const ElemDev& E = t.elems[C.elem_begin + k];
            for (int r = 0; r < E.nth; ++r) rcell[E.row + r] = k;
        }
        for (int R = 0; R < Nth; ++R)
            for (int c = 0; c < Nth; ++c) {
                const double a = std::fabs(W[(int64_t)R * Nth + c]);
                if (c == R || a == 0.) continue;
                wmin = (wmin == 0.) ? a : std::min(wmin, a);
                wmax = std::max(wmax, a);
                if (rcell[R] == rcell[c]) cmax[rcell[R]] = std::max(cmax[rcell[R]], a);
            }
        const double dxdy8 = t.colc[ci];
        for (int ij = 0; ij < C.nx * C.ny; ++ij) {
            const double swv = t.sw[C.node_off + ij];
            const double cw = dxdy8 * swv;
            uint8_t cls;
            if (!(std::fabs(swv) > kSmall)) {
                // cross-cell terms left out: the per-term loop when any own-cell term is kept
                bool any = false;
                for (int k = 0; k < ncell; ++k) any |= std::fabs(cw * cmax[k]) > kSmall;
                cls = any ? 2 : 0;
            } else if (wmax == 0.) {
                cls = 0;
            } else if (std::fabs(cw * wmin) > kSmall) {
                cls = 1;
            } else if (!(std::fabs(cw * wmax) > kSmall)) {
                cls = 0;
            } else {
                cls = 2;
            }
            scls[C.node_off + ij] = cls;
            ++pt->nodes[cls];
            if (cls == 1 && ij < 64) colfull[ci] |= 1ull << ij;
            if (cls == 2 && Nth <= 64) {
                // the exact FP64 test of every term of every row of the node
                const bool cross = std::fabs(swv) > kSmall;
                kbase[C.node_off + ij] = (int64_t)kmask.size();
                for (int R = 0; R < Nth; ++R) {
                    uint64_t mk = 0;
                    for (int c = 0; c < Nth; ++c) {
                        if (c == R || (!cross && rcell[c] != rcell[R])) continue;
                        if (std::fabs(cw * W[(int64_t)R * Nth + c]) > kSmall) mk |= 1ull << c;
                    }
                    kmask.push_back(mk);
                }
            }
        }
    }
    const int ncpl = (int)t.cpls.size();
    std::vector<double> mortc;
    pt->esc.assign(ncpl, 0);
    pt->etc.assign(ncpl, 0);
    pt->tested.assign(ncpl, 0);
    std::map<std::pair<int, std::vector<char>>, int> et_seen;   // (Et offset, zeroed entries) -> offset
    for (int e = 0; e < (int)t.elems.size(); ++e) {
        const ElemDev& E = t.elems[e];
        const ColDev& C = t.cols[E.col];
        for (int k = E.cpl_begin; k < E.cpl_end; ++k) {
            const CplDev& cp = t.cpls[k];
            const CplGeo& g = t.cgeo[k];
            const int n0 = (cp.face % 2 == 0) ? C.ny : C.nx;
            const int nes = g.m1 * n0, net = g.nth1 * E.nth;
            const double dc = t.cplc[k];
            std::vector<double> des(nes);
            for (int q = 0; q < nes; ++q) des[q] = dc * t.mort[cp.es + q];
            const double* et = t.mort.data() + cp.et;
            // an entry is removable when every product it takes part in is dropped
            std::vector<char> esz(nes, 0), etz(net, 0);
            std::vector<char> es_any(nes, 0), et_any(net, 0), es_kept(nes, 0), et_kept(net, 0);
            for (int q = 0; q < nes; ++q) {
                if (des[q] == 0.) continue;
                for (int b = 0; b < net; ++b) {
                    if (et[b] == 0.) continue;
                    const bool kept = std::fabs(des[q] * et[b]) > kBcTol;
                    es_any[q] = et_any[b] = 1;
                    if (kept) es_kept[q] = et_kept[b] = 1;
                }
            }
            for (int q = 0; q < nes; ++q) esz[q] = es_any[q] && !es_kept[q];
            for (int b = 0; b < net; ++b) etz[b] = et_any[b] && !et_kept[b];
            bool separable = true;
            for (int q = 0; q < nes && separable; ++q) {
                if (des[q] == 0.) continue;
                for (int b = 0; b < net; ++b) {
                    if (et[b] == 0.) continue;
                    const bool dropped = !(std::fabs(des[q] * et[b]) > kBcTol);
                    if (dropped != (esz[q] || etz[b])) {
                        separable = false;
                        break;
                    }
                }
            }
            if (!separable) {
                pt->tested[k] = 1;
                ++pt->ntested;
                continue;
            }
            pt->esc[k] = (int)mortc.size();
            for (int q = 0; q < nes; ++q) mortc.push_back(esz[q] ? 0. : des[q]);
            auto key = std::make_pair((int)cp.et, etz);
            auto f = et_seen.find(key);
            if (f != et_seen.end()) {
                pt->etc[k] = f->second;
            } else {
                pt->etc[k] = (int)mortc.size();
                for (int b = 0; b < net; ++b) mortc.push_back(etz[b] ? 0. : et[b]);
                et_seen.emplace(std::move(key), pt->etc[k]);
            }
        }
    }
    if (mortc.size() > (size_t)INT32_MAX) throw RtgError{RTG_ERR_ARG, "cleaned mortar table too large"};
    try {
        RTG_CUDA(cudaMalloc(&pt->d_scls, scls.size()));
        RTG_CUDA(cudaMemcpy(pt->d_scls, scls.data(), scls.size(), cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMalloc(&pt->d_colfull, sizeof(uint64_t) * std::max<size_t>(colfull.size(), 1)));
        if (!colfull.empty())
            RTG_CUDA(cudaMemcpy(pt->d_colfull, colfull.data(), sizeof(uint64_t) * colfull.size(),
                                cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMalloc(&pt->d_kbase, sizeof(int64_t) * kbase.size()));
        RTG_CUDA(cudaMemcpy(pt->d_kbase, kbase.data(), sizeof(int64_t) * kbase.size(), cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMalloc(&pt->d_kmask, sizeof(uint64_t) * std::max<size_t>(kmask.size(), 1)));
        if (!kmask.empty())
            RTG_CUDA(cudaMemcpy(pt->d_kmask, kmask.data(), sizeof(uint64_t) * kmask.size(), cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMalloc(&pt->d_mortc, sizeof(double) * std::max<size_t>(mortc.size(), 1)));
        if (!mortc.empty())
            RTG_CUDA(cudaMemcpy(pt->d_mortc, mortc.data(), sizeof(double) * mortc.size(), cudaMemcpyHostToDevice));
    } catch (...) {
        free_parity(pt);
        throw;
    }
    return pt;
}

// Tiled items of the FP32 path: consecutive cells of a column, at most
// kTileRows angular rows and kTileOut outputs per item, when the column's
// input, the item's W rows and its products fit in shared memory.


static size_t tile_smem_bytes(size_t vsize, int nth_col, int nij, int wcap, int M, int ncell) {
    const int nijp = (nij + 3) & ~3, Mp = (M + 3) & ~3;
    return vsize * ((size_t)nth_col * nijp + (size_t)wcap + (size_t)Mp * nijp) + sizeof(int) * (2 * ncell + 2) + 16;
}

// cap: per column, the largest number of angular rows of a tiled item;
// include: per column, whether the plan covers it (null: every column);
// par: the FP64 tiled path's tables (null: FP64 columns use the per-output
// kernels).
template <typename T>
static ApplyPlan* make_plan(const rtg_handle* h, const std::vector<int>* cap = nullptr,
                            const std::vector<char>* include = nullptr, int chunk64 = kChunk64,
                            const ParityTables* par = nullptr) {
    const HostTables& t = h->host;
    constexpr bool parity = sizeof(T) == 8;
    ApplyPlan* p = new ApplyPlan();
    std::vector<std::pair<int64_t, int4>> items[2];
    std::vector<std::pair<int64_t, TileItem>> tiles;
    std::vector<std::vector<TileCpl>> tile_cpl;   // coupling entries per tiled item
    std::vector<int32_t> slow;
    size_t need[2] = {0, 0};
    for (int ci = 0; ci < (int)t.cols.size(); ++ci) {
        if (include && !(*include)[ci]) continue;
        const ColDev& C = t.cols[ci];
        const int ncell = C.elem_end - C.elem_begin;
        const int nij = C.nx * C.ny;
        const int rows_cap = cap ? (*cap)[ci] : kTileRows;
        if ((!parity || par) && ncell <= kMaxCellsStaged) {
            // split the column into items of whole cells
            std::vector<TileItem> its;
            bool fits = true;
            int k = 0;
            std::vector<std::vector<TileCpl>> ents;
            std::vector<size_t> bytes;
            while (k < ncell && fits) {
                TileItem ti{ci, k, k, t.elems[C.elem_begin + k].row, 0, 0, 0, 0, 0, 0};
                int M = 0, ncp = 0;
                while (k < ncell) {
                    const ElemDev& E = t.elems[C.elem_begin + k];
                    const int nth = E.nth, nc = E.cpl_end - E.cpl_begin;
                    if (M > 0 && (M + nth > rows_cap || (M + nth) * nij > kTileOut || ncp + nc > kMaxItemCpl ||
                                  k - ti.cell_begin >= kMaxItemCells))
                        break;
                    M += nth;
                    ncp += nc;
                    ++k;
                }
                ti.cell_end = k;
                if (ncp > kMaxItemCpl) fits = false;
                std::vector<TileCpl> en;
                int tsz = 0, csz = 0;
                for (int q = ti.cell_begin; q < ti.cell_end; ++q) {
                    const ElemDev& E = t.elems[C.elem_begin + q];
                    for (int kk = E.cpl_begin; kk < E.cpl_end; ++kk) {
                        const CplGeo& g = t.cgeo[kk];
                        const CplDev& cp = t.cpls[kk];
                        TileCpl tc{};
                        tc.base = g.base;
                        tc.rowloc = E.row - ti.row0;
                        tc.nth = E.nth;
                        tc.toff = tsz;
                        tc.coff = csz;
                        tc.m1 = g.m1;
                        tc.nt1 = g.nth1;
                        tc.face = cp.face;
                        tc.n0 = (cp.face % 2 == 0) ? C.ny : C.nx;
                        tc.stride = g.stride;
                        tc.es = parity ? par->esc[kk] : cp.es;
                        tc.et = parity ? par->etc[kk] : cp.et;
                        tc.dc = (float)t.cplc[kk];
                        tc.k = kk;
                        tc.tested = parity ? par->tested[kk] : 0;
                        en.push_back(tc);
                        tsz += g.m1 * E.nth;
                        csz += tc.n0 * E.nth;
                    }
                }
                ti.ttot = tsz;
                ti.ctot = 0;
                for (int q = ti.cell_begin; q < ti.cell_end; ++q)
                    ti.ctot += boundary_nodes(C.nx, C.ny) * t.elems[C.elem_begin + q].nth;
                (void)csz;
                const int Mp = (M + 3) & ~3, nijp = (nij + 3) & ~3;
                // Fy and Ys are read and written four values at a time: keep
                // every region a multiple of 4 values from the aligned base
                ti.tsz = (tsz + 3) & ~3;
                ti.wcap = std::max(C.nth_col * Mp, ti.tsz + Mp * nijp);
                if ((ti.wcap & 3) || (ti.tsz & 3) || (nijp & 3))
                    throw RtgError{RTG_ERR_ARG, "tiled apply: unaligned shared-memory region"};
                const size_t b = tile_smem_bytes(sizeof(T), C.nth_col, nij, ti.wcap, M, ncell);
                if (b > kSmemBudget) fits = false;
                bytes.push_back(b);
                ents.push_back(std::move(en));
                its.push_back(ti);
            }
            if (fits) {
                for (size_t q = 0; q < its.size(); ++q) {
                    const TileItem& ti = its[q];
                    int M = 0;
                    for (int r = ti.cell_begin; r < ti.cell_end; ++r) M += t.elems[C.elem_begin + r].nth;
                    p->tile_smem = std::max(p->tile_smem, bytes[q]);
                    tiles.push_back({(int64_t)M * nij * (C.nth_col + C.nx + C.ny) + C.ndof, ti});
                    tile_cpl.push_back(std::move(ents[q]));
                }
                continue;
            }
        }
        const size_t sx = sizeof(T) * (size_t)C.ndof + sizeof(int) * (2 * ncell + 2) + 16;
        const size_t sw = (sizeof(T) + (parity ? sizeof(float) : 0)) * (size_t)C.nth_col * (C.nth_col | 1);
        if (sx > kSmemBudget || ncell > kMaxCellsStaged) {
            slow.push_back(ci);
            continue;
        }
        const int grp = (sx + sw <= kSmemBudget) ? 0 : 1;
        need[grp] = std::max(need[grp], grp == 0 ? sx + sw : sx);
        const int chunk = parity ? chunk64 : kChunk;
        const int nch = (C.ndof + chunk - 1) / chunk;
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
    std::vector<int> perm(tiles.size());
    for (size_t q = 0; q < perm.size(); ++q) perm[q] = (int)q;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return tiles[a].first > tiles[b].first; });
    std::vector<TileItem> tv;
    std::vector<TileCpl> ent;
    for (int q : perm) {
        TileItem ti = tiles[q].second;
        ti.cpl_begin = (int)ent.size();
        ent.insert(ent.end(), tile_cpl[q].begin(), tile_cpl[q].end());
        ti.cpl_end = (int)ent.size();
        tv.push_back(ti);
    }
    p->ntiles = (int)tv.size();
    p->par = parity ? par : nullptr;
    p->d_tiles = (TileItem*)up(tv.data(), sizeof(TileItem) * tv.size());
    p->d_tile_cpl = (TileCpl*)up(ent.data(), sizeof(TileCpl) * ent.size());
    return p;
}

static void free_plan(ApplyPlan* p) {
    if (!p) return;
    for (void* d : p->allocs) cudaFree(d);
    if (p->own_par) free_parity(p->par);
    delete p;
}

template <typename T>
static void set_plan_attributes(const ApplyPlan* p) {
    constexpr bool f64 = sizeof(T) == 8;
    raise_smem_limit((const void*)apply_col_kernel<T, T, f64>, std::max(p->g[0].smem, p->g[1].smem));
    if (p->ntiles) raise_smem_limit((const void*)apply_tiled_kernel<T, f64>, p->tile_smem);
}

template <typename T>
static void run_plan(const ApplyPlan* plan, const OpView<T>& v, const OpView<float>& v32, uint32_t flags, const T* x,
                     T* y, cudaStream_t s) {
    constexpr bool f64 = sizeof(T) == 8;
    RTG_LAUNCHED("a kernel before the apply");
    {
        if (plan->ntiles) {
            TileParity<T> tp{};
            if constexpr (f64) {
                tp.scls = plan->par->d_scls;
                tp.mortc = plan->par->d_mortc;
                tp.mortf = v32.mort;
                tp.Wf = v32.W;
                tp.colfull = plan->par->d_colfull;
                tp.kbase = plan->par->d_kbase;
                tp.kmask = plan->par->d_kmask;
            }
            apply_tiled_kernel<T, f64><<<plan->ntiles, kApplyThreads, plan->tile_smem, s>>>(
                v, tp, flags, plan->d_tiles, plan->d_tile_cpl, x, y), count_launch();
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                cudaFuncAttributes fa{};
                cudaFuncGetAttributes(&fa, apply_tiled_kernel<T, f64>);
                throw RtgError{RTG_ERR_CUDA, "launch of apply_tiled_kernel (items " + std::to_string(plan->ntiles) +
                                                 ", dynamic smem " + std::to_string(plan->tile_smem) + ", max dynamic " +
                                                 std::to_string(fa.maxDynamicSharedSizeBytes) + ", static " +
                                                 std::to_string(fa.sharedSizeBytes) + "): " + cudaGetErrorString(e)};
            }
        }
    }
    for (int grp = 0; grp < 2; ++grp) {
        const ApplyGroup& G = plan->g[grp];
        if (G.nitems) {
            apply_col_kernel<T, T, f64><<<G.nitems, kApplyThreads, G.smem, s>>>(v, v32.W, v32.mort, flags,
                                                                              G.d_items, G.stage_w, x, y), count_launch();
            RTG_LAUNCHED("apply_col_kernel");
        }
    }
    if (plan->nslow) {
        apply_global_kernel<T, T, f64><<<plan->nslow, kApplyThreads, 0, s>>>(v, v32.mort, flags, plan->d_slow, x, y), count_launch();
        RTG_LAUNCHED("apply_global_kernel");
    }
}

// Autotuner of the FP32 path: for every degree class of columns, time the
// class's items with each candidate row cap (one warm-up, best of three
// launches, CUDA events) and keep the fastest; then build the plan with the
// chosen cap per column.
static ApplyPlan* tune_plan32(rtg_handle* h, cudaStream_t s) {
    const HostTables& t = h->host;
    const int nc = (int)t.cols.size();
    auto pow2 = [](int n) {
        int b = 1;
        while (b < n) b <<= 1;
        return b;
    };
    std::map<std::tuple<int, int, int>, std::vector<int>> classes;
    for (int ci = 0; ci < nc; ++ci) {
        const ColDev& C = t.cols[ci];
        classes[std::make_tuple(C.nx, C.ny, pow2(C.nth_col))].push_back(ci);
    }
    float *x = nullptr, *y = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<int> cap(nc, kTileRows);
    std::vector<TuneRecord> recs;
    try {
        RTG_CUDA(cudaMalloc(&x, sizeof(float) * std::max<int64_t>(t.ndof, 1)));
        RTG_CUDA(cudaMalloc(&y, sizeof(float) * std::max<int64_t>(t.ndof, 1)));
        RTG_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * t.ndof, s));
        RTG_CUDA(cudaEventCreate(&e0));
        RTG_CUDA(cudaEventCreate(&e1));
        const uint32_t flags = RTG_SYSTEM | RTG_MASK_ROWS;
        for (const auto& kv : classes) {
            std::vector<char> inc(nc, 0);
            for (int ci : kv.second) inc[ci] = 1;
            TuneRecord r{std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first), kTileRows, {}};
            float best = 1e30f;
            for (int q = 0; q < kNumTuneCaps; ++q) {
                r.ns[q] = -1;
                std::vector<int> cq(nc, kTuneCaps[q]);
                ApplyPlan* p = make_plan<float>(h, &cq, &inc);
                try {
                    set_plan_attributes<float>(p);
                    run_plan<float>(p, h->v32, h->v32, flags, x, y, s);
                    float tbest = 1e30f;
                    for (int rep = 0; rep < 3; ++rep) {
                        RTG_CUDA(cudaEventRecord(e0, s));
                        run_plan<float>(p, h->v32, h->v32, flags, x, y, s);
                        RTG_CUDA(cudaEventRecord(e1, s));
                        RTG_CUDA(cudaEventSynchronize(e1));
                        float ms = 0.f;
                        RTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                        tbest = std::min(tbest, ms);
                    }
                    r.ns[q] = (int)(tbest * 1e6f);
                    // a larger cap must win by 3% to displace a smaller one
                    if (tbest < best * 0.97f) {
                        best = tbest;
                        r.cap = kTuneCaps[q];
                    }
                } catch (...) {
                    free_plan(p);
                    throw;
                }
                free_plan(p);
            }
            for (int ci : kv.second) cap[ci] = r.cap;
            recs.push_back(r);
        }
    } catch (...) {
        if (x) cudaFree(x);
        if (y) cudaFree(y);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        throw;
    }
    // a class timed alone sees an idle GPU: keep the tuned plan only if the
    // whole apply is faster with it than with the default item size
    ApplyPlan* tuned = make_plan<float>(h, &cap, nullptr);
    ApplyPlan* dflt = nullptr;
    try {
        dflt = make_plan<float>(h, nullptr, nullptr);
        float tt = 1e30f, td = 1e30f;
        for (ApplyPlan* p : {tuned, dflt}) {
            set_plan_attributes<float>(p);
            run_plan<float>(p, h->v32, h->v32, RTG_SYSTEM | RTG_MASK_ROWS, x, y, s);
            for (int rep = 0; rep < 3; ++rep) {
                RTG_CUDA(cudaEventRecord(e0, s));
                run_plan<float>(p, h->v32, h->v32, RTG_SYSTEM | RTG_MASK_ROWS, x, y, s);
                RTG_CUDA(cudaEventRecord(e1, s));
                RTG_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                RTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                (p == tuned ? tt : td) = std::min(p == tuned ? tt : td, ms);
            }
        }
        if (td < tt) {
            std::swap(tuned, dflt);
            for (TuneRecord& r : recs) r.cap = -r.cap;   // negative: class choice not used
        }
    } catch (...) {
        free_plan(tuned);
        free_plan(dflt);
        cudaFree(x);
        cudaFree(y);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    free_plan(dflt);
    cudaFree(x);
    cudaFree(y);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tuned->tuning = std::move(recs);
    return tuned;
}

// FP64 apply: columns that fit in shared memory run the tiled kernel with the
// drop rules resolved on the host (build_parity); the whole apply is timed
// with 16, 32 and 64 angular rows per tiled item (best of three after a
// warm-up) and the fastest plan is kept.
static ApplyPlan* tune_plan64(rtg_handle* h, cudaStream_t s) {
    const int64_t N = h->host.ndof;
    const int nc = (int)h->host.cols.size();
    double *x = nullptr, *y = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ApplyPlan* best = nullptr;
    float tbest = 1e30f;
    ParityTables* par = build_parity(h);
    auto release = [&] {
        if (x) cudaFree(x);
        if (y) cudaFree(y);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    try {
        RTG_CUDA(cudaMalloc(&x, sizeof(double) * std::max<int64_t>(N, 1)));
        RTG_CUDA(cudaMalloc(&y, sizeof(double) * std::max<int64_t>(N, 1)));
        RTG_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * N, s));
        RTG_CUDA(cudaEventCreate(&e0));
        RTG_CUDA(cudaEventCreate(&e1));
        for (int rows : {16, 32, 64}) {
            std::vector<int> cap(nc, rows);
            ApplyPlan* p = make_plan<double>(h, &cap, nullptr, kChunk64, par);
            float tt = 1e30f;
            try {
                set_plan_attributes<double>(p);
                run_plan<double>(p, h->v64, h->v32, RTG_SYSTEM | RTG_MASK_ROWS, x, y, s);
                for (int rep = 0; rep < 3; ++rep) {
                    RTG_CUDA(cudaEventRecord(e0, s));
                    run_plan<double>(p, h->v64, h->v32, RTG_SYSTEM | RTG_MASK_ROWS, x, y, s);
                    RTG_CUDA(cudaEventRecord(e1, s));
                    RTG_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    RTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    tt = std::min(tt, ms);
                }
            } catch (...) {
                free_plan(p);
                throw;
            }
            if (tt < tbest) {
                free_plan(best);
                best = p;
                tbest = tt;
            } else {
                free_plan(p);
            }
        }
    } catch (...) {
        free_plan(best);
        free_parity(par);
        release();
        throw;
    }
    release();
    best->own_par = true;
    return best;
}

int apply_tuning(rtg_handle* h, int32_t* out, int cap_rows, cudaStream_t s) {
    if (!h->plan32) {
        h->plan32 = tune_plan32(h, s);
        set_plan_attributes<float>(h->plan32);
    }
    const auto& rec = h->plan32->tuning;
    const int n = (int)rec.size();
    for (int i = 0; i < std::min(n, cap_rows); ++i) {
        int32_t* o = out + (size_t)i * (4 + kNumTuneCaps);
        o[0] = rec[i].nx;
        o[1] = rec[i].ny;
        o[2] = rec[i].nthb;
        o[3] = rec[i].cap;
        for (int q = 0; q < kNumTuneCaps; ++q) o[4 + q] = rec[i].ns[q];
    }
    return n;
}

void free_apply_plans(rtg_handle* h) {
    free_plan(h->plan64);
    free_plan(h->plan32);
    h->plan64 = h->plan32 = nullptr;
}

template <typename T>
void launch_apply(const rtg_handle* hc, const OpView<T>& v, uint32_t flags, const T* x, T* y,
                  cudaStream_t s) {
    rtg_handle* h = const_cast<rtg_handle*>(hc);
    constexpr bool f64 = sizeof(T) == 8;
    ApplyPlan*& plan = f64 ? h->plan64 : h->plan32;
    if (!plan) {
        plan = f64 ? tune_plan64(h, s) : tune_plan32(h, s);
        set_plan_attributes<T>(plan);
    }
    run_plan<T>(plan, v, h->v32, flags, x, y, s);
}

template void launch_apply<double>(const rtg_handle*, const OpView<double>&, uint32_t, const double*,
                                   double*, cudaStream_t);
template void launch_apply<float>(const rtg_handle*, const OpView<float>&, uint32_t, const float*,
                                  float*, cudaStream_t);

void launch_interior_mask(const rtg_handle* h, uint8_t* mask, cudaStream_t s) {
    interior_mask_kernel<<<h->v64.nelem, 128, 0, s>>>(h->v64, mask), count_launch();
    RTG_CUDA(cudaGetLastError());
}

void launch_mask_vector(const rtg_handle* h, int part, const double* x, double* out, cudaStream_t s) {
    mask_vector_kernel<<<h->v64.nelem, 128, 0, s>>>(h->v64, part, x, out), count_launch();
    RTG_CUDA(cudaGetLastError());
}

void launch_weight_forcing(const rtg_handle* h, const double* f, double* out, cudaStream_t s) {
    weight_forcing_kernel<<<h->v64.nelem, 128, 0, s>>>(h->v64, f, out), count_launch();
    RTG_CUDA(cudaGetLastError());
}

}  // namespace rtg

// Matrix-free application of the RT DG operator and the small vector kernels
// around it.  A spatial column is the unit of work: the column's DOFs are
// contiguous (cell-major, then i, j, a), the scattering block is dense over
// the column's angular nodes and diagonal in the spatial node (i, j), and the
// streaming terms stay inside one element.
//
// Main path (apply_tiled_kernel): one CTA per column (or per work item of a
// column) stages the column's input in shared memory transposed to
// [angular row R][spatial node ij] and walks the column's items: scattering
// product from shared memory in 4 x 4 register tiles, factorised inflow face
// fluxes, then every output DOF written in global order.  FP32 plans may hand
// the scattering product to scat_tc_kernel (tcgen05 tensor cores, TF32 hi/lo
// split).  The plan shape (rows per item, items per CTA, launches per
// shared-memory class, tensor cores or not) is autotuned per handle
// (tune_plan).  Columns too large for the tiled path use apply_col_kernel
// (per-output chunks from shared memory) or apply_global_kernel (operands
// read from global memory).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <future>
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
// One CTA per column: the column's input is staged once, transposed
// (Xs[row][ij]), and the CTA walks the column's items.  An item is whole
// cells [cell_begin, cell_end), i.e. the rectangle of angular rows
// R0 .. R0+M-1 times all nij spatial nodes.  The scattering of the item is the
// product Y[m][ij] = sum_c W[R0+m][c] X[c][ij] over all Nth angular nodes of
// the column; it runs from shared memory with 4 x 4 register tiles (16 FMAs
// per eight loaded values).  The epilogue adds extinction, streaming and face
// terms and writes y in global order.  The inflow face fluxes of the item's
// elements are factorised per coupling (T[jj][r] = sum_a Et[a][r]
// x_nbr[jj][a], then sum_jj Es[jj][q] T[jj][r]) and accumulated into Fy
// before the epilogue; T and Fy reuse the W region.  Every global -> shared
// copy is a cp.async, so a staging loop has all its loads in flight.
// Shared memory: Xs[Nth][nijp] | column table | cell rows and flags | item
// region: WsT[Nth][Mp] (later T | Fy[Mp][nijp]) | Ys[Mp][nijp] |
// row table[Mp][kRowVals] | row -> cell.  Without the product (the
// tensor-core path takes it) a CTA may hold any run of items of its column,
// down to one, and Xs holds only the current item's rows.
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
    int M;                    // angular rows of the item
    int cpl0;                 // coupling index of the item's first entry
};

// One coupling of a tiled item: where its neighbour line is, its mortars,
// and its offsets in the two flux phases.  FP64: es and et index the cleaned
// tables (dcoeff*Es and Et); k is the coupling, tested marks a coupling summed
// term by term.
struct TileCpl {
    int64_t base;             // neighbour line: x[base + jj*stride + a]
    int nth, toff;            // the element's angular nodes; first value of its T block
    int m1, nt1, n0, face;
    int stride, es, et;
    float dc;
    int k, tested;
    int diag;                 // bit 0: Es diagonal (m1 == n0, off-diagonal entries exactly 0); bit 1: Et diagonal
    int pad;                  // 64 bytes: copied in 16-byte pieces
};
constexpr int kMaxItemCpl = 96;
static_assert(sizeof(TileCpl) == 64, "coupling records are copied in 16-byte pieces");

// Host-built tables of the FP64 tiled path.
// Scattering classes of a spatial node (the reference keeps an off-diagonal
// term of the (M - S) block iff |value| > 1e-14):
//   0 no term kept, 1 every term kept, 2 the terms with |W| >= the node's
//   threshold kept (cross-cell terms included), 3 own-cell terms only
//   (|wx wy sigma| <= 1e-14), each tested on its own.
// Classes 1 and 2 read the product; its tiles mask W by the threshold.
template <typename T>
struct TileParity {
    const uint8_t* scls = nullptr;   // per spatial node: class 0..3
    const T* mortc = nullptr;        // cleaned dcoeff*Es and Et per coupling
    const float* mortf = nullptr;    // FP32 copy of the mortars (tested couplings)
    const float* Wf = nullptr;       // FP32 copy of W (class-3 nodes)
    const uint64_t* colfull = nullptr;   // per column: bit ij set when node ij reads the product (ij < 64)
    // per spatial node: bits of the smallest |W| whose term is kept (class 1:
    // 0, every term; classes 0 and 3: +inf bits, none).  For w >= 0 the order
    // of the IEEE bit patterns is the order of the values, so the test is an
    // integer compare.
    const uint64_t* thr = nullptr;
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

// sum_jj Es[jj][q] T[jj][r] of one coupling at face node q, row r; with a
// diagonal Es its one nonzero term, and with Es and Et both diagonal (no T
// formed) Es[q][q] (Et[r][r] x_line[q][r]): the same roundings as the full sums,
// whose other terms are exact zeros
template <typename T, typename Cpl>
__device__ __forceinline__ T face_sum(const Cpl& en, const T* Es, const T* Et, const T* Tb, const T* x, int q, int r) {
    if (en.diag == 3) return Es[q * en.n0 + q] * (Et[r * en.nth + r] * x[en.base + (int64_t)q * en.stride + r]);
    if (en.diag & 1) return Es[q * en.n0 + q] * Tb[en.toff + q * en.nth + r];
    T sacc = T(0);
    for (int jj = 0; jj < en.m1; ++jj) sacc = fma(Es[jj * en.n0 + q], Tb[en.toff + jj * en.nth + r], sacc);
    return sacc;
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

// values of the per-row table: dxdydth/8 * wth_r, dx dth/4, dy dth/4, wth_r,
// wth_r sin, wth_r cos, ThF_0..3 of the row's cell
constexpr int kRowVals = 10;

// threads of a tiled CTA: FP32 items are latency bound (more warps per SM),
// FP64 ones register bound
template <typename T>
__host__ __device__ constexpr int tiled_threads() { return sizeof(T) == 8 ? 256 : 512; }

// values of the per-column table: kw and sw per node, LGL weights in x and y,
// the two derivative tables
__host__ __device__ __forceinline__ int col_table_size(int nx, int ny) {
    return (2 * nx * ny + nx + ny + nx * nx + ny * ny + 3) & ~3;
}
// ints before the item region: per cell its first row, flags, first coupling
// and angular table offset, per row its cell; padded to 32 bytes
__host__ __device__ __forceinline__ int col_int_words(int ncell, int nth_col) {
    return (4 * ncell + 2 + nth_col + 7) & ~7;
}

// kProduct = false: the tensor-core kernel does the scattering product (FP32),
// so the CTA neither stages W nor runs the product and fits three per SM
template <typename T, bool kParity, bool kProduct = true>
__global__ void __launch_bounds__(tiled_threads<T>(), sizeof(T) == 8 ? 3 : (kProduct ? 2 : 3))
apply_tiled_kernel(OpView<T> v, TileParity<T> par, uint32_t flags, const int4* __restrict__ groups,
                   const TileItem* __restrict__ items, const TileCpl* __restrict__ cpl_ent, const T* __restrict__ x,
                   T* __restrict__ y) {
    extern __shared__ double2 smt4[];
    __shared__ __align__(16) TileCpl sc[kMaxItemCpl];
    __shared__ float s_rcp[kMaxNodes + 1];    // 1/n rounded to float
    T* smt = reinterpret_cast<T*>(smt4);
    if (v.stop && *v.stop) return;
    const int4 grp = groups[blockIdx.x];      // column, first item, end item
    const int ci = grp.x;
    if (v.skip && v.skip[ci]) return;
    const ColDev C = v.cols[ci];
    const ApplyFlags fl = decode(flags);
    const bool scat = kProduct && fl.scat;
    const int nij = C.nx * C.ny, Nth = C.nth_col, ncell = C.elem_end - C.elem_begin;
    const int nijp = (nij + 3) & ~3, Nthp = (Nth + 3) & ~3;
    // with the product every row of x is staged once per column; without it
    // (tensor-core path) each item stages its own rows (grp.w: the most rows
    // of an item of the group, a multiple of 4)
    const int xrows = kProduct ? Nth : grp.w;
    T* Xs = smt;                                                  // [xrows][nijp]
    T* colt = Xs + (size_t)xrows * nijp;                          // column table
    T* rowt = colt + col_table_size(C.nx, C.ny);                  // [Nthp][kRowVals]
    int* crow = reinterpret_cast<int*>(rowt + (size_t)Nthp * kRowVals);   // [ncell+1] first row; crow[ncell] = Nth
    int* cflg = crow + ncell + 1;                                          // [ncell] element flags
    int* ccpl = cflg + ncell;                                              // [ncell+1] first coupling
    int* cang = ccpl + ncell + 1;                                          // [ncell] angular table offset
    int* rcell = cang + ncell;                                             // [Nth] cell of each row
    T* ireg = reinterpret_cast<T*>(crow + col_int_words(ncell, Nth));    // item region
    const T* kwn = colt;
    const T* swn = colt + nij;
    const T* wxs = colt + 2 * nij;
    const T* wys = wxs + C.nx;
    const T* Gxs = wys + C.ny;
    const T* Gys = Gxs + C.nx * C.nx;
    // per-cell tables and the column table
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) {
        const ElemDev E = v.elems[C.elem_begin + k];
        crow[k] = E.row;
        cflg[k] = E.flags;
        ccpl[k] = E.cpl_begin;
        cang[k] = E.ang;
        if (k == ncell - 1) {
            crow[ncell] = Nth;
            ccpl[ncell] = E.cpl_end;
        }
        for (int r = 0; r < E.nth; ++r) rcell[E.row + r] = k;
    }
    if (threadIdx.x <= kMaxNodes) s_rcp[threadIdx.x] = threadIdx.x ? __frcp_rn((float)threadIdx.x) : 0.f;
    {
        const T* Gx = v.G + gofs(C.nx);
        const T* Gy = v.G + gofs(C.ny);
        const int o1 = nij, o2 = 2 * nij, o3 = o2 + C.nx, o4 = o3 + C.ny, o5 = o4 + C.nx * C.nx;
        const int tot = o5 + C.ny * C.ny;
        for (int q = threadIdx.x; q < tot; q += blockDim.x) {
            const T* src = q < o1   ? v.kw + C.node_off + q
                           : q < o2 ? v.sw + C.node_off + (q - o1)
                           : q < o3 ? v.lglw + C.nx * kMaxNodes + (q - o2)
                           : q < o4 ? v.lglw + C.ny * kMaxNodes + (q - o3)
                           : q < o5 ? Gx + (q - o4)
                                    : Gy + (q - o5);
            cp_async_small<sizeof(T)>(colt + q, src);
        }
    }
    __syncthreads();
    const T* xc = x + C.dof_off;
    // stage x transposed: Xs[row][ij]; pad columns are zero (d grows per
    // thread, so the cell index k only moves forward)
    if constexpr (kProduct) {
        int k = 0;
        for (int d = threadIdx.x; d < C.ndof; d += blockDim.x) {
            while (d >= nij * crow[k + 1]) ++k;
            const int nth = crow[k + 1] - crow[k];
            const int l = d - nij * crow[k];
            const int ij = small_div(l, s_rcp[nth]);
            cp_async_small<sizeof(T)>(Xs + (crow[k] + l - ij * nth) * nijp + ij, xc + d);
        }
        if (nijp != nij)
            for (int t = threadIdx.x; t < Nth * (nijp - nij); t += blockDim.x)
                Xs[(t / (nijp - nij)) * nijp + nij + t % (nijp - nij)] = T(0);
    }
    // the column's row table
    for (int R = threadIdx.x; R < Nth; R += blockDim.x) {
        const int k = rcell[R];
        const int e = C.elem_begin + k;
        const int r = R - crow[k], nth = crow[k + 1] - crow[k];
        const T* A = v.ang + cang[k];
        T* rw = rowt + R * kRowVals;
        const T ar = A[r];
        rw[0] = v.econst[4 * e] * ar;
        rw[1] = v.econst[4 * e + 1];
        rw[2] = v.econst[4 * e + 2];
        rw[3] = ar;
        rw[4] = A[nth + r];
        rw[5] = A[2 * nth + r];
#pragma unroll
        for (int F = 0; F < 4; ++F) rw[6 + F] = A[(3 + F) * nth + r];
    }
    const T* Wg = v.W + v.W_off[C.sig];
    const T small = T(kSmall);
    const T dxdy8 = v.colc[ci];
    const float rny = __frcp_rn((float)C.ny);
    T* yc = y + C.dof_off;
    for (int iq = grp.y; iq < grp.z; ++iq) {
        const TileItem it = items[iq];
        const int M = it.M, Mp = (M + 3) & ~3;
        T* WsT = ireg;                                // [Nth][Mp]
        T* Ys = WsT + (size_t)it.wcap;                // [Mp][nijp]
        T* Tb = WsT;                                  // after the product: T
        T* Fy = WsT + it.tsz;                         //                    Fy[Mp][nijp]
        // the item's couplings (64-byte records, four 16-byte copies each)
        {
            const int nent = it.cpl_end - it.cpl_begin;
            const char* src = reinterpret_cast<const char*>(cpl_ent + it.cpl_begin);
            char* dst = reinterpret_cast<char*>(sc);
            for (int q = threadIdx.x; q < nent * (int)(sizeof(TileCpl) / 16); q += blockDim.x)
                cp_async16(dst + 16 * q, src + 16 * q);
        }
        if (scat) {
            // W^T staged by rows of W^T, so consecutive threads read consecutive values
            const T* WTg = v.WT + v.W_off[C.sig];
            const float rMp = __frcp_rn((float)Mp);
            for (int t = threadIdx.x; t < Nth * Mp; t += blockDim.x) {
                const int c = small_div(t, rMp), m = t - c * Mp;
                // FP64: the diagonal joins the extinction term in the epilogue
                const bool use = m < M && !(kParity && c == it.row0 + m);
                if (use)
                    cp_async_small<sizeof(T)>(WsT + t, WTg + (int64_t)c * Nth + it.row0 + m);
                else
                    WsT[t] = T(0);
            }
        }
        if constexpr (!kProduct) {
            // the item's rows of x (its DOFs are contiguous: whole cells),
            // row R at Xs[R - row0]; the product does not run, so the pad
            // columns are never read
            int k = it.cell_begin;
            for (int d = nij * it.row0 + threadIdx.x; d < nij * (it.row0 + M); d += blockDim.x) {
                while (d >= nij * crow[k + 1]) ++k;
                const int nth = crow[k + 1] - crow[k];
                const int l = d - nij * crow[k];
                const int ij = small_div(l, s_rcp[nth]);
                cp_async_small<sizeof(T)>(Xs + (crow[k] - it.row0 + l - ij * nth) * nijp + ij, xc + d);
            }
        }
        cp_async_wait_all();
        __syncthreads();
        if (scat) {
            const int tm = Mp / 4, tn = nijp / 4, ntile = tm * tn;
            const float rtn = __frcp_rn((float)tn);
            // FP64: nodes of classes 1 and 2 read the product
            const uint64_t fullm = kParity ? (nij <= 64 ? par.colfull[ci] : ~0ull) : ~0ull;
            // ks adjacent lanes share a 4 x 4 tile, each summing every ks-th
            // angular node, so that items of a few rows still keep every warp
            // busy; the partial sums meet through shuffles (ks = 1, 2, 4 or 8,
            // the same for the whole CTA, so the loop below is uniform)
            int ks = 1;
            while (ks < 8 && ntile * ks * 2 <= (int)blockDim.x) ks *= 2;
            const int slot = threadIdx.x & (ks - 1);
            const int per = blockDim.x / ks;
            for (int tb0 = 0; tb0 < ntile; tb0 += per) {
                const int tile = tb0 + (int)threadIdx.x / ks;
                const int tq = tile < ntile ? small_div(tile, rtn) : 0;
                const int m0 = 4 * tq, j0 = 4 * (tile - tq * tn);
                const bool act = tile < ntile && !(kParity && j0 < 64 && !((fullm >> j0) & 0xFull));
                T acc[4][4];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
                if (act) {
                    if constexpr (kParity) {
                        // the drop rule per (row, node): keep w iff bits(|w|) >= thr(node)
                        // (integer compares: no work for the slow FP64 pipe)
                        unsigned long long tb[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            tb[j] = j0 + j < nij ? par.thr[C.node_off + j0 + j] : 0x7FF0000000000000ull;
#pragma unroll 2
                        for (int c = slot; c < Nth; c += ks) {
                            T wv[4], xa[4];
                            load4(WsT + c * Mp + m0, wv);
                            load4(Xs + c * nijp + j0, xa);
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                // the dropped terms' W zeroed by an integer mask of its bits
                                // (no FP64 select)
                                const unsigned long long wbits = (unsigned long long)__double_as_longlong((double)wv[i]);
                                const unsigned long long wb = wbits & 0x7FFFFFFFFFFFFFFFull;
#pragma unroll
                                for (int j = 0; j < 4; ++j) {
                                    const unsigned long long keep = wb >= tb[j] ? ~0ull : 0ull;
                                    acc[i][j] = fma(__longlong_as_double((long long)(wbits & keep)), xa[j], acc[i][j]);
                                }
                            }
                        }
                    } else {
#pragma unroll 4
                        for (int c = slot; c < Nth; c += ks) {
                            T wv[4], xa[4];
                            load4(WsT + c * Mp + m0, wv);
                            load4(Xs + c * nijp + j0, xa);
#pragma unroll
                            for (int i = 0; i < 4; ++i)
#pragma unroll
                                for (int j = 0; j < 4; ++j) acc[i][j] = fma(wv[i], xa[j], acc[i][j]);
                        }
                    }
                }
                // reduce-scatter over the ks lanes of the tile: each step
                // halves the partial sums a lane holds (it keeps one half and
                // adds its partner's copy of it), so lane s ends with 16/ks
                // finished outputs from index base (row-major in the tile)
                T a[16];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) a[4 * i + j] = acc[i][j];
                int base = 0;
                if (ks >= 2) {
                    const bool up = slot & 1;
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const T keep = up ? a[q + 8] : a[q], send = up ? a[q] : a[q + 8];
                        a[q] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
                    }
                    base += up ? 8 : 0;
                }
                if (ks >= 4) {
                    const bool up = slot & 2;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const T keep = up ? a[q + 4] : a[q], send = up ? a[q] : a[q + 4];
                        a[q] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
                    }
                    base += up ? 4 : 0;
                }
                if (ks >= 8) {
                    const bool up = slot & 4;
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const T keep = up ? a[q + 2] : a[q], send = up ? a[q] : a[q + 2];
                        a[q] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
                    }
                    base += up ? 2 : 0;
                }
                if (act) {
                    const int cnt = 16 / ks;
#pragma unroll
                    for (int q = 0; q < 16; ++q)
                        if (q < cnt) Ys[(m0 + ((base + q) >> 2)) * nijp + j0 + ((base + q) & 3)] = a[q];
                }
            }
        }
        __syncthreads();
        // inflow face fluxes of the item's elements into Fy (the W region is free)
        if (fl.bc) {
            for (int t = threadIdx.x; t < Mp * nijp; t += blockDim.x) Fy[t] = T(0);
            // T[jj][r] = sum_a Et[a][r] x_line[jj][a] of every coupling: one warp
            // per coupling, its lanes over (jj, r).  Couplings whose Es and Et
            // are both diagonal (conforming neighbours) have no T: the flux
            // phase reads their line values directly.  With a diagonal Et the
            // sum is its one nonzero term (the others add exact zeros).
            {
                const int lane = threadIdx.x & 31, nwarp = (int)blockDim.x >> 5;
                const int nent = it.cpl_end - it.cpl_begin;
                for (int c = (int)threadIdx.x >> 5; c < nent; c += nwarp) {
                    const TileCpl& en = sc[c];
                    if ((kParity && en.tested) || en.diag == 3) continue;   // tested: summed term by term below
                    const int nth = en.nth, nt1 = en.nt1, cnt = en.m1 * nth;
                    const bool dt = en.diag & 2;
                    const T* Et = (kParity ? par.mortc : v.mort) + en.et;
                    for (int q = lane; q < cnt; q += 32) {
                        const int jj = small_div(q, s_rcp[nth]), r = q - jj * nth;
                        const T* xl = x + en.base + (int64_t)jj * en.stride;
                        T acc = T(0);
                        if (dt) {
                            acc = Et[r * nth + r] * xl[r];
                        } else {
                            // the loads of up to 8 line values issued before their sum
#pragma unroll
                            for (int a = 0; a < 8; ++a)
                                if (a < nt1) acc = fma(Et[a * nth + r], xl[a], acc);
                            for (int a = 8; a < nt1; ++a) acc = fma(Et[a * nth + r], xl[a], acc);
                        }
                        Tb[en.toff + q] = acc;
                    }
                }
            }
            __syncthreads();
            // one thread per (boundary node, row): the element's couplings on the
            // node's faces in a fixed order, so the sum is deterministic
            {
                const float rM = __frcp_rn((float)M);
                for (int t = threadIdx.x; t < it.ctot; t += blockDim.x) {
                    const int f = small_div(t, rM), m = t - f * M;
                    const int R = it.row0 + m, k = rcell[R];
                    const int r = R - crow[k];
                    const int c0 = ccpl[k] - it.cpl0, c1 = ccpl[k + 1] - it.cpl0;
                    int i, j;
                    boundary_node(f, C.nx, C.ny, i, j);
                    T acc = T(0);
                    for (int c = c0; c < c1; ++c) {
                        const TileCpl& en = sc[c];
                        const int F = en.face;
                        const bool on = (F == 0 && i == C.nx - 1) || (F == 1 && j == C.ny - 1) ||
                                        (F == 2 && i == 0) || (F == 3 && j == 0);
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
                                acc += face_sum(en, Es, par.mortc + en.et, Tb, x, q, r);
                            }
                        } else {
                            const T* Es = v.mort + en.es;
                            const T sacc = face_sum(en, Es, v.mort + en.et, Tb, x, q, r);
                            acc = fma(T(en.dc), sacc, acc);
                        }
                    }
                    Fy[m * nijp + i * C.ny + j] = acc;
                }
            }
            __syncthreads();
        }
        const int d0 = nij * it.row0, d1 = nij * (it.row0 + M);
        int k = it.cell_begin;
        for (int d = d0 + threadIdx.x; d < d1; d += blockDim.x) {
            while (d >= nij * crow[k + 1]) ++k;
            const int nth = crow[k + 1] - crow[k];
            const int l = d - nij * crow[k];
            const int ij = small_div(l, s_rcp[nth]), r = l - ij * nth;
            const int i = small_div(ij, rny), j = ij - i * C.ny;
            const int flg = cflg[k];
            if (fl.mask_rows && bdry_node(flg >> 4, i, j, C.nx, C.ny)) {
                if constexpr (kProduct) yc[d] = T(0);   // tensor-core path: y was zeroed
                continue;
            }
            const int R = crow[k] + r;
            const int m = R - it.row0;   // row within the item
            const int xr0 = kProduct ? R : m;   // row of Xs
            const T* rw = rowt + R * kRowVals;
            const T xself = Xs[xr0 * nijp + ij];
            const T mterm = rw[0] * kwn[ij];
            T acc = T(0);
            if constexpr (kParity) {
                if (scat) {
                    const int node = C.node_off + ij;
                    const T swv = swn[ij];
                    const T cw = dxdy8 * swv;
                    const int cls = par.scls[node];
                    T s = T(0);
                    if (cls == 1 || cls == 2) {
                        s = Ys[m * nijp + ij];
                    } else if (cls == 3) {
                        // own-cell terms only, some kept: test each one
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
                if (scat) acc = -dxdy8 * swn[ij] * Ys[m * nijp + ij];
                if (fl.mass) acc += mterm * xself;
            }
            if (fl.ic) {
                const T* xr = Xs + xr0 * nijp;
                T t1 = T(0), t2 = T(0);
                const T* gy = Gys + j * C.ny;
                for (int jj = 0; jj < C.ny; ++jj) t1 += gy[jj] * xr[i * C.ny + jj];
                const T* gx = Gxs + i * C.nx;
                for (int ii = 0; ii < C.nx; ++ii) t2 += gx[ii] * xr[ii * C.ny + j];
                const T ic = rw[1] * wxs[i] * rw[4] * t1 + rw[2] * wys[j] * rw[5] * t2;
                acc += T(fl.ic_sign) * ic;
            }
            if (fl.bc && (i == 0 || j == 0 || i == C.nx - 1 || j == C.ny - 1)) {
                acc += Fy[m * nijp + ij];
                // outflow faces: the diagonal term (rt/boundary_convection_matrix.py:276-346)
                for (int F = 0; F < 4; ++F) {
                    if (!(flg & (1 << F))) continue;
                    const bool on = (F == 0 && i == C.nx - 1) || (F == 1 && j == C.ny - 1) || (F == 2 && i == 0) ||
                                    (F == 3 && j == 0);
                    if (!on) continue;
                    const T dc = (F % 2 == 0) ? rw[2] : rw[1];
                    const T w = (F % 2 == 0) ? wys[j] : wxs[i];
                    const T val = dc * w * rw[3] * rw[6 + F];
                    if (!kParity || tabs(val) > T(kBcTol)) acc += val * xself;
                }
            }
            // tensor-core path: the scattering kernel adds its part to the
            // same zeroed y concurrently; two terms on zero sum the same in
            // either order
            if constexpr (kProduct)
                yc[d] = acc;
            else
                atomicAdd(yc + d, acc);
        }
        // the next item overwrites the couplings and the item region
        __syncthreads();
    }
}

// ------------------------------------------------- tensor-core scattering
// FP32 scattering product on the 5th-generation tensor cores: one CTA per
// (column, tile of 128 angular rows): D[m][ij] = sum_c W[R0+m][c] X[c][ij],
// then y[R0+m, ij] += -(dx dy / 8) sw_ij D[m][ij] by an atomic add: the
// caller zeroes y and the tiled kernel adds the other terms concurrently on
// another stream (exactly two terms on zero, so the sum does not depend on
// their order); rows of inflow-boundary nodes stay zero.
// Each value is split into TF32 hi + lo parts (hi = round-to-nearest TF32,
// lo = value - hi, exact in FP32) and D accumulates A_lo B_hi + A_hi B_lo +
// A_hi B_hi with tcgen05.mma (kind::tf32, M = 128, N = nij padded to 16,
// K = 8 per instruction, one issuing thread) in tensor memory.  The K axis
// (the column's angular nodes) is walked in chunks of kTcK: W's hi/lo tile of
// the chunk is built once per handle on the host in the shared-memory image
// and arrives with one bulk copy (cp.async.bulk, completion counted on an
// mbarrier); x is gathered with cp.async straight into its place and split
// in place.  tcgen05.commit signals the chunk's MMAs on a second mbarrier
// before the operands are restaged.  Operands use the canonical K-major
// layout without swizzle: 8-row x 16-byte core matrices, K-adjacent ones 128
// bytes apart, 8-row groups kTcK/4 * 128 bytes apart.
constexpr int kTcThreads = 256;
constexpr int kTcM = 128;
constexpr int kTcK = 32;
constexpr int kTcTileFloats = 2 * kTcM * kTcK;   // hi and lo of one W tile

struct TcItem {
    int col, row0, rows, pad;
    int64_t wtile;   // first W tile of the item's row tile (tiles of its chunks follow)
};

__host__ __device__ __forceinline__ int tc_np(int nij) { return nij <= 16 ? 16 : (nij + 15) & ~15; }
__host__ __device__ __forceinline__ int tc_tmem_cols(int np) {
    int c = 32;
    while (c < np) c <<= 1;
    return c;
}

// float offset of (row, k) in the canonical layout, and its inverse
__host__ __device__ __forceinline__ int tc_off(int row, int k) {
    return (row >> 3) * (kTcK / 4) * 32 + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}
__device__ __forceinline__ void tc_pos(int p, int& row, int& k) {
    row = (p / ((kTcK / 4) * 32)) * 8 + ((p >> 2) & 7);
    k = ((p >> 5) % (kTcK / 4)) * 4 + (p & 3);
}

__device__ __forceinline__ uint64_t tc_desc(const float* p) {
    const uint64_t a = (uint64_t)__cvta_generic_to_shared(p);
    const uint64_t lbo = 128, sbo = (kTcK / 4) * 128;
    return ((a >> 4) & 0x3FFFull) | (((lbo >> 4) & 0x3FFFull) << 16) | (((sbo >> 4) & 0x3FFFull) << 32) |
           (1ull << 46);   // descriptor version 1, base offset 0, no swizzle
}

__device__ __forceinline__ float tf32_hi(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// bounded wait for the completion of phase `parity` of an mbarrier
__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t parity) {
    uint32_t done = 0;
    for (int spin = 0; spin < (1 << 22) && !done; ++spin)
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mb), "r"(parity)
            : "memory");
    return done != 0;
}

__global__ void __launch_bounds__(kTcThreads)
scat_tc_kernel(OpView<float> v, uint32_t flags, const TcItem* __restrict__ items, const float* __restrict__ wtc,
               const float* __restrict__ x, float* __restrict__ y, int* __restrict__ status) {
    extern __shared__ __align__(128) float tsm[];
    __shared__ __align__(8) uint64_t mbar_mma, mbar_ld;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    __shared__ int s_crow[kMaxCellsStaged + 1];
    __shared__ int s_cflg[kMaxCellsStaged];
    if (v.stop && *v.stop) return;
    const TcItem it = items[blockIdx.x];
    if (v.skip && v.skip[it.col]) return;
    const ColDev C = v.cols[it.col];
    const ApplyFlags fl = decode(flags);
    const int nij = C.nx * C.ny, Nth = C.nth_col, ncell = C.elem_end - C.elem_begin;
    const int np = tc_np(nij), ncols = tc_tmem_cols(np);
    float* As = tsm;                       // W tile: hi [kTcM x kTcK] | lo
    float* Bh = As + kTcTileFloats;        // x: hi [np x kTcK] | lo
    float* Bl = Bh + np * kTcK;
    int* rcell = reinterpret_cast<int*>(Bl + np * kTcK);   // [Nth] cell of each row
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) {
        const ElemDev E = v.elems[C.elem_begin + k];
        s_crow[k] = E.row;
        s_cflg[k] = E.flags;
        if (k == ncell - 1) s_crow[ncell] = Nth;
        for (int r = 0; r < E.nth; ++r) rcell[E.row + r] = k;
    }
    const uint32_t mb_mma = (uint32_t)__cvta_generic_to_shared(&mbar_mma);
    const uint32_t mb_ld = (uint32_t)__cvta_generic_to_shared(&mbar_ld);
    if (threadIdx.x == 0) {
        s_abort = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb_mma) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb_ld) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s_tmem);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    // kind::tf32: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2),
    // both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(np >> 3) << 17) |
                           ((uint32_t)(kTcM >> 4) << 24);
    const float* xc = x + C.dof_off;
    const uint32_t as_addr = (uint32_t)__cvta_generic_to_shared(As);
    const int nchunk = (Nth + kTcK - 1) / kTcK;
    for (int ch = 0; ch < nchunk; ++ch) {
        const int c0 = ch * kTcK;
        if (threadIdx.x == 0) {
            // the chunk's W tile (hi and lo, in the shared-memory image) in one bulk copy
            const float* src = wtc + (it.wtile + ch) * (int64_t)kTcTileFloats;
            const uint32_t bytes = kTcTileFloats * sizeof(float);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb_ld), "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    as_addr),
                "l"(src), "r"(bytes), "r"(mb_ld)
                : "memory");
        }
        // x gathered into its place: consecutive threads fill consecutive
        // shared-memory words (B[ij][k] = x at angular row c0 + k, node ij)
        for (int p = threadIdx.x; p < np * kTcK; p += blockDim.x) {
            int n, k;
            tc_pos(p, n, k);
            const int c = c0 + k;
            if (n < nij && c < Nth) {
                const int kc = rcell[c];
                const int nth = s_crow[kc + 1] - s_crow[kc];
                cp_async_small<4>(Bh + p, xc + nij * s_crow[kc] + n * nth + (c - s_crow[kc]));
            } else {
                Bh[p] = 0.f;
            }
        }
        cp_async_wait_all();
        __syncthreads();
        for (int p = threadIdx.x; p < np * kTcK; p += blockDim.x) {
            const float xv = Bh[p];
            const float h = tf32_hi(xv);
            Bh[p] = h;
            Bl[p] = xv - h;
        }
        // generic-proxy writes -> visible to the tensor cores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            if (!mbar_wait(mb_ld, (uint32_t)(ch & 1))) {
                s_abort = 1;
            } else {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const float* Ah = As;
                const float* Al = As + kTcM * kTcK;
#pragma unroll
                for (int s = 0; s < kTcK / 8; ++s) {
                    const int o = 64 * s;   // two K-adjacent core matrices per K = 8
                    tc_mma(tmem, tc_desc(Al + o), tc_desc(Bh + o), idesc, ch > 0 || s > 0);
                    tc_mma(tmem, tc_desc(Ah + o), tc_desc(Bl + o), idesc, 1);
                    tc_mma(tmem, tc_desc(Ah + o), tc_desc(Bh + o), idesc, 1);
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 mb_mma)
                             : "memory");
            }
        }
        __syncthreads();
        if (s_abort) break;
        // the chunk's MMAs have read the operands before they are restaged
        if (!mbar_wait(mb_mma, (uint32_t)(ch & 1))) s_abort = 1;
        __syncthreads();
        if (s_abort) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (s_abort) {
        if (threadIdx.x == 0 && status) atomicExch(status, RTG_ERR_TIMEOUT);
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (rows), columns
        // [h np/2, (h+1) np/2) with h = w / 4
        const int q = warp & 3, h = warp >> 2;
        const int m = 32 * q + lane, R = it.row0 + m;
        const bool valid = m < it.rows;
        const int kc = valid ? rcell[R] : 0;
        const int nth = s_crow[kc + 1] - s_crow[kc];
        const int r = R - s_crow[kc];
        const float dxdy8 = v.colc[it.col];
        const int half = np / 2;
        for (int cb = h * half; cb < (h + 1) * half; cb += 8) {
            uint32_t d[8];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
                "tcgen05.wait::ld.sync.aligned;"
                : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7])
                : "r"(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)cb)
                : "memory");
            if (!valid) continue;
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
                const int ij = cb + jj;
                if (ij >= nij) break;
                const int i = ij / C.ny, j = ij % C.ny;
                if (fl.mask_rows && bdry_node(s_cflg[kc] >> 4, i, j, C.nx, C.ny)) continue;
                const int64_t dof = C.dof_off + (int64_t)nij * s_crow[kc] + (int64_t)ij * nth + r;
                atomicAdd(y + dof, -dxdy8 * v.sw[C.node_off + ij] * __uint_as_float(d[jj]));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// W tiles of the tensor-core path for one signature: per row tile of 128 and
// chunk of kTcK columns, hi then lo in the shared-memory image (zero outside
// W); hi rounds to the nearest TF32 value (ties away from zero, the rounding
// of cvt.rna), lo = w - hi.
static void tc_w_tiles(const float* W, int n, std::vector<float>& out) {
    const int mt = (n + kTcM - 1) / kTcM, kc = (n + kTcK - 1) / kTcK;
    const size_t base = out.size();
    out.resize(base + (size_t)mt * kc * kTcTileFloats, 0.f);
    for (int t = 0; t < mt; ++t)
        for (int ch = 0; ch < kc; ++ch) {
            float* blk = out.data() + base + ((size_t)t * kc + ch) * kTcTileFloats;
            for (int m = 0; m < kTcM; ++m)
                for (int k = 0; k < kTcK; ++k) {
                    const int R = t * kTcM + m, c = ch * kTcK + k;
                    if (R >= n || c >= n) continue;
                    const float w = W[(size_t)R * n + c];
                    uint32_t b;
                    std::memcpy(&b, &w, 4);
                    uint32_t hb = b;
                    if ((b & 0x7F800000u) != 0x7F800000u) hb = (b + 0x1000u) & 0xFFFFE000u;
                    float hi;
                    std::memcpy(&hi, &hb, 4);
                    blk[tc_off(m, k)] = hi;
                    blk[kTcM * kTcK + tc_off(m, k)] = w - hi;
                }
        }
}

static size_t tc_smem_bytes(int nij, int nth_col) {
    return sizeof(float) * ((size_t)kTcTileFloats + 2 * (size_t)tc_np(nij) * kTcK) + sizeof(int) * (size_t)nth_col +
           16;
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
// FP64 chunks of the per-output kernels are smaller: that path is FP64-pipe
// bound, and smaller chunks balance the SMs.
constexpr int kChunk64 = 256;

struct ApplyGroup {
    int4* d_items = nullptr;
    int nitems = 0;
    size_t smem = 0;
    int stage_w = 0;
};

constexpr int kTileRows = 64;       // default row cap (before tuning)
constexpr int kTileOut = 2048;
// launches of the tiled kernel: groups that fit 4, 3, 2 or 1 CTAs per SM
constexpr int kSmemClasses = 4;

// Shape of a tiled plan: angular rows per item, items per CTA (0: the whole
// column), and whether the CTAs are launched per shared-memory class (each
// launch with its own dynamic shared memory) or in one launch.
struct PlanShape {
    int rows = kTileRows;
    int gcap = 0;
    int split = 0;
    int tc = 0;    // FP32: scattering of the tiled columns on the tensor cores (scat_tc_kernel),
                   // CTAs heaviest first; 2: the same with the columns of one angular mesh in
                   // consecutive CTAs
};

// One timed plan shape of the autotuner (time in ns, -1: not run).
struct TuneRecord {
    PlanShape shape;
    int chosen, ns, items, groups, launches;
};

// Tables of the FP64 tiled path (drop rules resolved on the host): the
// scattering class of every spatial node and the cleaned mortar products of
// every coupling.
struct ParityTables {
    uint8_t* d_scls = nullptr;
    double* d_mortc = nullptr;
    uint64_t* d_colfull = nullptr;
    uint64_t* d_thr = nullptr;
    std::vector<int> esc, etc;     // per coupling: offsets of dcoeff*Es and Et in the cleaned table
    std::vector<char> tested;      // per coupling: summed term by term
    std::vector<uint8_t> diag;     // per coupling: cleaned Es (bit 0) / Et (bit 1) diagonal
    int64_t nodes[4] = {0, 0, 0, 0};   // nodes per scattering class
    int64_t ntested = 0;
};

struct ApplyPlan {
    ApplyGroup g[2];            // 0: input and W staged; 1: input staged, W read through L2
    int32_t* d_slow = nullptr;
    int nslow = 0;
    TileItem* d_tiles = nullptr;   // tiled items, grouped per CTA
    TileCpl* d_tile_cpl = nullptr; // their coupling entries
    int ntiles = 0;
    int4* d_tgroups = nullptr;     // per CTA: column, first item, end item
    int tg_begin[kSmemClasses + 1] = {};   // CTAs of launch q: [tg_begin[q], tg_begin[q+1])
    size_t tg_smem[kSmemClasses] = {};     // dynamic shared memory of launch q
    size_t tile_smem = 0;                  // the largest of them
    TcItem* d_tc = nullptr;                // tensor-core scattering CTAs
    float* d_wtc = nullptr;                // their W tiles (hi/lo, shared-memory image)
    int ntc = 0;
    size_t tc_smem = 0;
    int* d_status = nullptr;               // RTG_ERR_TIMEOUT if a wait of scat_tc_kernel gave up
    // tensor-core plans: y is zeroed, then the tiled kernels (on the caller's
    // stream) and scat_tc_kernel (on side) add their parts concurrently
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int64_t ndof = 0;
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
    cudaFree(pt->d_thr);
    delete pt;
}

// 1 when an m x n mortar block (row-major) is square with exact zeros off the
// diagonal
template <typename V>
static uint8_t mortar_diag(const V* b, int m, int n) {
    if (m != n) return 0;
    for (int a = 0; a < m; ++a)
        for (int c = 0; c < n; ++c)
            if (a != c && b[a * n + c] != V(0)) return 0;
    return 1;
}
// the same for a block with the entries flagged in z zeroed
static uint8_t mortar_diag_clean(const double* b, const std::vector<char>& z, int m, int n) {
    if (m != n) return 0;
    for (int a = 0; a < m; ++a)
        for (int c = 0; c < n; ++c)
            if (a != c && !z[a * n + c] && b[a * n + c] != 0.) return 0;
    return 1;
}

// Resolves the FP64 drop rules of the tiled path on the host, with the same
// FP64 products and comparisons the per-term path makes.
//  * node class: |fl(cw w)| grows with |w|, so the smallest and largest
//    nonzero off-diagonal |W| entries decide whether every, no or some
//    scattering term of the node is kept (cross-cell terms only where
//    |wx wy sigma| > 1e-14, rt/preconditioner_matrix.py:450-495); for "some"
//    the kept terms are exactly those with |w| >= t, t the smallest double
//    with |fl(cw t)| > 1e-14, found by stepping from 1e-14 / |cw|;
//  * coupling: the terms dropped by |dcoeff Es Et| <= 1e-15 must be exactly
//    the products with a set of Es entries or a set of Et entries; then those
//    entries are zeroed in copies of dcoeff*Es and Et
//    (rt/boundary_convection_matrix.py:258-524).
static ParityTables* build_parity(const rtg_handle* h) {
    const HostTables& t = h->host;
    ParityTables* pt = new ParityTables();
    std::vector<uint8_t> scls((size_t)std::max(t.nnodes, 1), 0);
    constexpr uint64_t kInfBits = 0x7FF0000000000000ull;
    std::vector<uint64_t> colfull(t.cols.size(), 0);
    std::vector<uint64_t> thr((size_t)std::max(t.nnodes, 1), kInfBits);
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
                cls = any ? 3 : 0;
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
            if ((cls == 1 || cls == 2) && ij < 64) colfull[ci] |= 1ull << ij;
            if (cls == 1) {
                thr[C.node_off + ij] = 0;
            } else if (cls == 2) {
                // smallest t >= 0 with |fl(cw t)| > 1e-14 (fl(|cw| t) is monotone in t)
                const double acw = std::fabs(cw);
                double tt = kSmall / acw;
                auto kept = [&](double w) { return std::fabs(cw * w) > kSmall; };
                for (int it = 0; it < 64 && kept(tt); ++it) tt = std::nextafter(tt, 0.);
                for (int it = 0; it < 64 && !kept(tt); ++it) tt = std::nextafter(tt, HUGE_VAL);
                if (!kept(tt) || kept(std::nextafter(tt, 0.)))
                    throw RtgError{RTG_ERR_ARG, "drop-rule threshold not found"};
                uint64_t bits;
                std::memcpy(&bits, &tt, sizeof(bits));
                thr[C.node_off + ij] = bits;
            }
        }
    }
    const int ncpl = (int)t.cpls.size();
    std::vector<double> mortc;
    pt->esc.assign(ncpl, 0);
    pt->etc.assign(ncpl, 0);
    pt->tested.assign(ncpl, 0);
    pt->diag.assign(ncpl, 0);
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
            pt->diag[k] = mortar_diag(mortc.data() + pt->esc[k], g.m1, n0) |
                          (mortar_diag_clean(et, etz, g.nth1, E.nth) << 1);
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
        RTG_CUDA(cudaMalloc(&pt->d_thr, sizeof(uint64_t) * thr.size()));
        RTG_CUDA(cudaMemcpy(pt->d_thr, thr.data(), sizeof(uint64_t) * thr.size(), cudaMemcpyHostToDevice));
        RTG_CUDA(cudaMalloc(&pt->d_mortc, sizeof(double) * std::max<size_t>(mortc.size(), 1)));
        if (!mortc.empty())
            RTG_CUDA(cudaMemcpy(pt->d_mortc, mortc.data(), sizeof(double) * mortc.size(), cudaMemcpyHostToDevice));
    } catch (...) {
        free_parity(pt);
        throw;
    }
    return pt;
}

// Tiled items: consecutive cells of a column, at most `rows` angular rows and
// kTileOut outputs per item.  A CTA takes a group of consecutive items of one
// column (gcap items, 0: all of them) and stages the column's input once.
// Shared memory of a group: the column part (input, column table, cell
// rows and flags) and the largest item region of its items.
// xrows: rows of x staged (the column's nth_col with the product, the most
// rows of an item of the group without it)
static size_t tile_col_bytes(size_t vsize, int nth_col, int nx, int ny, int ncell, int xrows) {
    const int nijp = (nx * ny + 3) & ~3, nthp = (nth_col + 3) & ~3;
    return vsize * ((size_t)xrows * nijp + (size_t)col_table_size(nx, ny) + (size_t)nthp * kRowVals) +
           sizeof(int) * col_int_words(ncell, nth_col) + 16;
}
static size_t tile_item_bytes(size_t vsize, int nx, int ny, int wcap, int M) {
    const int nijp = (nx * ny + 3) & ~3, Mp = (M + 3) & ~3;
    return vsize * ((size_t)wcap + (size_t)Mp * nijp);
}

// Dynamic shared memory that lets q CTAs of the tiled kernel share an SM,
// for q = 4, 3, 2, 1 (index 0..3).
template <typename T, bool kProduct>
static void smem_class_limits(size_t lim[kSmemClasses]) {
    int dev = 0, per_sm = 0, resv = 0;
    RTG_CUDA(cudaGetDevice(&dev));
    RTG_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    RTG_CUDA(cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    cudaFuncAttributes fa{};
    RTG_CUDA(cudaFuncGetAttributes(&fa, apply_tiled_kernel<T, sizeof(T) == 8, kProduct>));
    // CTAs per SM that registers and threads allow
    int maxb = 0;
    RTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, apply_tiled_kernel<T, sizeof(T) == 8, kProduct>,
                                                           tiled_threads<T>(), 0));
    for (int q = 0; q < kSmemClasses; ++q) {
        const int per = kSmemClasses - q;
        const long long l = (long long)per_sm / per - resv - (long long)fa.sharedSizeBytes;
        lim[q] = per > maxb ? 0 : (size_t)std::max(0ll, std::min(l, (long long)kSmemBudget));
    }
}

// cap: per column, the largest number of angular rows of a tiled item;
// include: per column, whether the plan covers it (null: every column);
// par: the FP64 tiled path's tables (null: FP64 columns use the per-output
// kernels); gcap, split: see PlanShape.
template <typename T>
static ApplyPlan* make_plan(const rtg_handle* h, const std::vector<int>* cap = nullptr,
                            const std::vector<char>* include = nullptr, int chunk64 = kChunk64,
                            const ParityTables* par = nullptr, int gcap = 0, int split = 0, int tc = 0) {
    const HostTables& t = h->host;
    constexpr bool parity = sizeof(T) == 8;
    if (parity) tc = 0;
    std::vector<std::pair<int64_t, TcItem>> tcv;
    std::map<int, int64_t> sig_tile;   // signature -> its first W tile
    std::vector<float> wtiles;
    ApplyPlan* p = new ApplyPlan();
    std::vector<std::pair<int64_t, int4>> items[2];
    struct GroupRec {
        int64_t cost;
        size_t smem;
        int col;
        int xrows;   // tensor-core path: x rows staged (the most rows of an item)
        std::vector<TileItem> its;
        std::vector<std::vector<TileCpl>> ents;
    };
    std::vector<GroupRec> groups;
    std::vector<int32_t> slow;
    size_t need[2] = {0, 0};
    for (int ci = 0; ci < (int)t.cols.size(); ++ci) {
        if (include && !(*include)[ci]) continue;
        const ColDev& C = t.cols[ci];
        const int ncell = C.elem_end - C.elem_begin;
        const int nij = C.nx * C.ny;
        const int rows_cap = cap ? (*cap)[ci] : kTileRows;
        if ((!parity || par) && ncell <= kMaxCellsStaged) {
            // split the column into items of whole cells; halve the rows per
            // item (down to 4) until every item fits next to the staged column
            std::vector<TileItem> its;
            std::vector<size_t> ibytes;
            std::vector<int64_t> icost;
            std::vector<std::vector<TileCpl>> ents;
            // column part of the shared memory with x rows xr
            auto colb = [&](int xr) { return tile_col_bytes(sizeof(T), C.nth_col, C.nx, C.ny, ncell, xr); };
            bool fits = false;
            for (int rcap = rows_cap; rcap > 0 && !fits; rcap = rcap > 4 ? rcap / 2 : 0) {
                its.clear();
                ibytes.clear();
                icost.clear();
                ents.clear();
                fits = true;
                int k = 0;
                while (k < ncell && fits) {
                    TileItem ti{ci, k, k, t.elems[C.elem_begin + k].row, 0, 0, 0, 0, 0, 0, 0,
                                t.elems[C.elem_begin + k].cpl_begin};
                    int M = 0, ncp = 0;
                    while (k < ncell) {
                        const ElemDev& E = t.elems[C.elem_begin + k];
                        const int nth = E.nth, nc = E.cpl_end - E.cpl_begin;
                        if (M > 0 && (M + nth > rcap || (M + nth) * nij > kTileOut || ncp + nc > kMaxItemCpl))
                            break;
                        M += nth;
                        ncp += nc;
                        ++k;
                    }
                    ti.cell_end = k;
                    ti.M = M;
                    if (ncp > kMaxItemCpl) fits = false;
                    std::vector<TileCpl> en;
                    int tsz = 0;
                    for (int q = ti.cell_begin; q < ti.cell_end; ++q) {
                        const ElemDev& E = t.elems[C.elem_begin + q];
                        for (int kk = E.cpl_begin; kk < E.cpl_end; ++kk) {
                            const CplGeo& g = t.cgeo[kk];
                            const CplDev& cp = t.cpls[kk];
                            TileCpl tc{};
                            tc.base = g.base;
                            tc.nth = E.nth;
                            tc.toff = tsz;
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
                            if (parity) {
                                tc.diag = tc.tested ? 0 : par->diag[kk];
                            } else {
                                // the FP32 tables are the FP32 roundings of these
                                std::vector<float> es32(g.m1 * tc.n0), et32(g.nth1 * E.nth);
                                for (size_t q = 0; q < es32.size(); ++q) es32[q] = (float)t.mort[cp.es + q];
                                for (size_t q = 0; q < et32.size(); ++q) et32[q] = (float)t.mort[cp.et + q];
                                tc.diag = mortar_diag(es32.data(), g.m1, tc.n0) |
                                          (mortar_diag(et32.data(), g.nth1, E.nth) << 1);
                            }
                            en.push_back(tc);
                            tsz += g.m1 * E.nth;
                        }
                    }
                    ti.ttot = tsz;
                    ti.ctot = boundary_nodes(C.nx, C.ny) * M;
                    const int Mp = (M + 3) & ~3, nijp = (nij + 3) & ~3;
                    // Fy and Ys are read and written four values at a time: keep
                    // every region a multiple of 4 values from the aligned base
                    ti.tsz = (tsz + 3) & ~3;
                    // without the scattering product (tensor-core path) the region holds T and Fy only
                    ti.wcap = tc ? ti.tsz + Mp * nijp : std::max(C.nth_col * Mp, ti.tsz + Mp * nijp);
                    if ((ti.wcap & 3) || (ti.tsz & 3) || (nijp & 3))
                        throw RtgError{RTG_ERR_ARG, "tiled apply: unaligned shared-memory region"};
                    ibytes.push_back(tile_item_bytes(sizeof(T), C.nx, C.ny, ti.wcap, M));
                    icost.push_back((int64_t)M * nij * (C.nth_col + C.nx + C.ny) + C.ndof);
                    ents.push_back(std::move(en));
                    its.push_back(ti);
                }
                for (size_t q = 0; q < its.size() && fits; ++q)
                    if (colb(tc ? (its[q].M + 3) & ~3 : C.nth_col) + ibytes[q] > kSmemBudget) fits = false;
                if (tc && tc_smem_bytes(nij, C.nth_col) > kSmemBudget) fits = false;
            }
            if (fits) {
                if (tc) {
                    auto its_ = sig_tile.find(C.sig);
                    if (its_ == sig_tile.end()) {
                        const int n = C.nth_col;
                        std::vector<float> wf((size_t)n * n);
                        for (size_t q = 0; q < wf.size(); ++q) wf[q] = (float)t.W[t.W_off[C.sig] + q];
                        const int64_t first = (int64_t)(wtiles.size() / kTcTileFloats);
                        tc_w_tiles(wf.data(), n, wtiles);
                        its_ = sig_tile.emplace(C.sig, first).first;
                    }
                    const int kc = (C.nth_col + kTcK - 1) / kTcK;
                    for (int r0 = 0; r0 < C.nth_col; r0 += kTcM)
                        tcv.push_back({(int64_t)std::min(kTcM, C.nth_col - r0) * C.nth_col * tc_np(nij),
                                       TcItem{ci, r0, std::min(kTcM, C.nth_col - r0), 0,
                                              its_->second + (int64_t)(r0 / kTcM) * kc}});
                }
                const size_t per = gcap > 0 ? (size_t)gcap : its.size();
                for (size_t q0 = 0; q0 < its.size(); q0 += per) {
                    GroupRec g{0, 0, ci, 0, {}, {}};
                    size_t ib = 0;
                    for (size_t q = q0; q < std::min(its.size(), q0 + per); ++q) {
                        g.cost += icost[q];
                        ib = std::max(ib, ibytes[q]);
                        if (tc) g.xrows = std::max(g.xrows, (its[q].M + 3) & ~3);
                        g.its.push_back(its[q]);
                        g.ents.push_back(std::move(ents[q]));
                    }
                    g.smem = colb(tc ? g.xrows : C.nth_col) + ib;
                    groups.push_back(std::move(g));
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
    // CTAs: heaviest first within each launch; launches by shared-memory
    // class, fewest CTAs per SM first (split), or all in one
    size_t lim[kSmemClasses];
    if (split && !groups.empty()) {
        if (tc)
            smem_class_limits<T, false>(lim);
        else
            smem_class_limits<T, true>(lim);
    } else {
        for (int q = 0; q < kSmemClasses; ++q) lim[q] = kSmemBudget;
    }
    auto cls = [&](size_t b) {
        for (int q = 0; q < kSmemClasses; ++q)
            if (b <= lim[q]) return q;
        return kSmemClasses - 1;
    };
    std::vector<int> perm(groups.size());
    for (size_t q = 0; q < perm.size(); ++q) perm[q] = (int)q;
    // launch order: class 3 (one CTA per SM) first, then 2, 1, 0
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) {
        const int ca = cls(groups[a].smem), cb2 = cls(groups[b].smem);
        if (ca != cb2) return ca > cb2;
        return groups[a].cost > groups[b].cost;
    });
    std::vector<TileItem> tv;
    std::vector<TileCpl> ent;
    std::vector<int4> tg;
    int counts[kSmemClasses] = {};
    for (int q : perm) {
        GroupRec& g = groups[q];
        const int c = cls(g.smem);
        const int first = (int)tv.size();
        for (size_t i = 0; i < g.its.size(); ++i) {
            TileItem ti = g.its[i];
            ti.cpl_begin = (int)ent.size();
            ent.insert(ent.end(), g.ents[i].begin(), g.ents[i].end());
            ti.cpl_end = (int)ent.size();
            tv.push_back(ti);
        }
        tg.push_back(make_int4(g.col, first, (int)tv.size(), g.xrows));
        const int slot = kSmemClasses - 1 - c;   // launch index
        counts[slot]++;
        p->tg_smem[slot] = std::max(p->tg_smem[slot], g.smem);
        p->tile_smem = std::max(p->tile_smem, g.smem);
    }
    p->tg_begin[0] = 0;
    for (int q = 0; q < kSmemClasses; ++q) p->tg_begin[q + 1] = p->tg_begin[q] + counts[q];
    p->ntiles = (int)tv.size();
    p->par = parity ? par : nullptr;
    p->d_tiles = (TileItem*)up(tv.data(), sizeof(TileItem) * tv.size());
    p->d_tile_cpl = (TileCpl*)up(ent.data(), sizeof(TileCpl) * ent.size());
    p->d_tgroups = (int4*)up(tg.data(), sizeof(int4) * tg.size());
    if (tc >= 2) {
        // columns of one angular mesh read the same W tiles: their CTAs run
        // next to each other (meshes by total cost, heaviest first), so that
        // the tiles come from L2 after the first read
        std::map<int, int64_t> sig_cost;
        for (auto& pr : tcv) sig_cost[t.cols[pr.second.col].sig] += pr.first;
        std::stable_sort(tcv.begin(), tcv.end(), [&](auto& a, auto& b) {
            const int sa = t.cols[a.second.col].sig, sb = t.cols[b.second.col].sig;
            const int64_t ca = sig_cost[sa], cb = sig_cost[sb];
            if (ca != cb) return ca > cb;
            if (sa != sb) return sa < sb;
            return a.second.row0 < b.second.row0;
        });
    } else {
        std::stable_sort(tcv.begin(), tcv.end(), [](auto& a, auto& b) { return a.first > b.first; });
    }
    std::vector<TcItem> tci;
    for (auto& pr : tcv) {
        tci.push_back(pr.second);
        const ColDev& C = t.cols[pr.second.col];
        p->tc_smem = std::max(p->tc_smem, tc_smem_bytes(C.nx * C.ny, C.nth_col));
    }
    p->ntc = (int)tci.size();
    p->ndof = t.ndof;
    if (p->ntc) {
        RTG_CUDA(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
        RTG_CUDA(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
        RTG_CUDA(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
    }
    p->d_tc = (TcItem*)up(tci.data(), sizeof(TcItem) * tci.size());
    p->d_wtc = (float*)up(wtiles.data(), sizeof(float) * wtiles.size());
    p->d_status = (int*)up(nullptr, 0);
    RTG_CUDA(cudaMemset(p->d_status, 0, sizeof(int)));
    return p;
}

static void free_plan(ApplyPlan* p) {
    if (!p) return;
    if (p->side) cudaStreamDestroy(p->side);
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    for (void* d : p->allocs) cudaFree(d);
    if (p->own_par) free_parity(p->par);
    delete p;
}

template <typename T>
static void set_plan_attributes(const ApplyPlan* p) {
    constexpr bool f64 = sizeof(T) == 8;
    raise_smem_limit((const void*)apply_col_kernel<T, T, f64>, std::max(p->g[0].smem, p->g[1].smem));
    if (p->ntiles) {
        if (p->ntc)
            raise_smem_limit((const void*)apply_tiled_kernel<T, f64, false>, p->tile_smem);
        else
            raise_smem_limit((const void*)apply_tiled_kernel<T, f64>, p->tile_smem);
    }
    if (p->ntc) raise_smem_limit((const void*)scat_tc_kernel, p->tc_smem);
}

template <typename T>
static void run_plan(const ApplyPlan* plan, const OpView<T>& v, const OpView<float>& v32, uint32_t flags, const T* x,
                     T* y, cudaStream_t s) {
    constexpr bool f64 = sizeof(T) == 8;
    RTG_LAUNCHED("a kernel before the apply");
    // tensor-core plan: zero y; the scattering runs on the side stream while
    // the tiled kernels run here (both add into y)
    const bool tc_run = !f64 && plan->ntc && (flags & (RTG_SYSTEM | RTG_SCAT));
    if (plan->ntc) RTG_CUDA(cudaMemsetAsync(y, 0, sizeof(T) * (size_t)plan->ndof, s));
    if (tc_run) {
        RTG_CUDA(cudaEventRecord(plan->ev_fork, s));
        RTG_CUDA(cudaStreamWaitEvent(plan->side, plan->ev_fork, 0));
        if constexpr (!f64) {
            scat_tc_kernel<<<plan->ntc, kTcThreads, plan->tc_smem, plan->side>>>(v, flags, plan->d_tc, plan->d_wtc, x,
                                                                                  y, plan->d_status),
                count_launch();
            RTG_LAUNCHED("scat_tc_kernel");
        }
        RTG_CUDA(cudaEventRecord(plan->ev_join, plan->side));
    }
    if (plan->ntiles) {
        TileParity<T> tp{};
        if constexpr (f64) {
            tp.scls = plan->par->d_scls;
            tp.mortc = plan->par->d_mortc;
            tp.mortf = v32.mort;
            tp.Wf = v32.W;
            tp.colfull = plan->par->d_colfull;
            tp.thr = plan->par->d_thr;
        }
        for (int q = 0; q < kSmemClasses; ++q) {
            const int n = plan->tg_begin[q + 1] - plan->tg_begin[q];
            if (!n) continue;
            const int4* grp = plan->d_tgroups + plan->tg_begin[q];
            if (plan->ntc)
                apply_tiled_kernel<T, f64, false><<<n, tiled_threads<T>(), plan->tg_smem[q], s>>>(
                    v, tp, flags, grp, plan->d_tiles, plan->d_tile_cpl, x, y), count_launch();
            else
                apply_tiled_kernel<T, f64><<<n, tiled_threads<T>(), plan->tg_smem[q], s>>>(
                    v, tp, flags, grp, plan->d_tiles, plan->d_tile_cpl, x, y), count_launch();
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                cudaFuncAttributes fa{};
                cudaFuncGetAttributes(&fa, apply_tiled_kernel<T, f64>);
                throw RtgError{RTG_ERR_CUDA, "launch of apply_tiled_kernel (CTAs " + std::to_string(n) +
                                                 ", dynamic smem " + std::to_string(plan->tg_smem[q]) +
                                                 ", max dynamic " + std::to_string(fa.maxDynamicSharedSizeBytes) +
                                                 ", static " + std::to_string(fa.sharedSizeBytes) +
                                                 "): " + cudaGetErrorString(e)};
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
    if (tc_run) RTG_CUDA(cudaStreamWaitEvent(s, plan->ev_join, 0));
}

static int plan_launches(const ApplyPlan* p) {
    int n = (p->g[0].nitems > 0) + (p->g[1].nitems > 0) + (p->nslow > 0) + (p->ntc > 0);
    for (int q = 0; q < kSmemClasses; ++q) n += p->tg_begin[q + 1] > p->tg_begin[q];
    return n;
}

// Builds the plan of one shape (FP64: with the host-resolved drop rules).
template <typename T>
static ApplyPlan* shape_plan(rtg_handle* h, const PlanShape& sh, const ParityTables* par) {
    std::vector<int> cap(h->host.cols.size(), sh.rows);
    return make_plan<T>(h, &cap, nullptr, kChunk64, par, sh.gcap, sh.split, sh.tc);
}

template <typename T>
static const OpView<T>& view_of(const rtg_handle* h) {
    if constexpr (sizeof(T) == 8)
        return h->v64;
    else
        return h->v32;
}

// Times a plan: one warm-up, best of three whole applies (CUDA events); a
// tensor-core plan whose waits gave up throws.
template <typename T>
static float time_plan(rtg_handle* h, ApplyPlan* p, const T* x, T* y, cudaEvent_t e0, cudaEvent_t e1,
                       cudaStream_t s) {
    set_plan_attributes<T>(p);
    run_plan<T>(p, view_of<T>(h), h->v32, RTG_SYSTEM | RTG_MASK_ROWS, x, y, s);
    float tt = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        RTG_CUDA(cudaEventRecord(e0, s));
        run_plan<T>(p, view_of<T>(h), h->v32, RTG_SYSTEM | RTG_MASK_ROWS, x, y, s);
        RTG_CUDA(cudaEventRecord(e1, s));
        RTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        RTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        tt = std::min(tt, ms);
    }
    if (p->ntc) {
        int st = 0;
        RTG_CUDA(cudaMemcpy(&st, p->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        if (st) {
            h->poisoned = true;
            throw RtgError{RTG_ERR_TIMEOUT, "scat_tc_kernel: a wait for the tensor cores gave up"};
        }
    }
    return tt;
}

// Autotuner of the apply: every plan shape of the candidate list (rows per
// item 16/32/64, one CTA per column or per item, one launch or one per
// shared-memory class, FP32: with or without the tensor-core scattering) is
// built and the whole apply timed; the fastest plan is kept.
template <typename T>
static ApplyPlan* tune_plan(rtg_handle* h, cudaStream_t s) {
    constexpr bool f64 = sizeof(T) == 8;
    const int64_t N = h->host.ndof;
    T *x = nullptr, *y = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ApplyPlan* best = nullptr;
    float tbest = 1e30f;
    int ibest = -1;
    ParityTables* par = f64 ? build_parity(h) : nullptr;
    std::vector<TuneRecord> recs;
    auto release = [&] {
        if (x) cudaFree(x);
        if (y) cudaFree(y);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    try {
        RTG_CUDA(cudaMalloc(&x, sizeof(T) * std::max<int64_t>(N, 1)));
        RTG_CUDA(cudaMalloc(&y, sizeof(T) * std::max<int64_t>(N, 1)));
        RTG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * N, s));
        RTG_CUDA(cudaEventCreate(&e0));
        RTG_CUDA(cudaEventCreate(&e1));
        std::vector<PlanShape> shapes;
        for (int rows : {16, 32, 64})
            for (int gcap : {0, 1})
                for (int split : {0, 1}) shapes.push_back(PlanShape{rows, gcap, split, 0});
        // tensor-core scattering (FP32): one CTA per column, items of 32 or 64
        // rows, the scattering CTAs of one angular mesh next to each other
        // (one CTA per item ties with these on the two-scatterer problem, and
        // the heaviest-first order of the scattering CTAs is 1.7 % slower there;
        // both are left out of the list, rtg_apply_shape can still pin them)
        if (!f64)
            for (int rows : {32, 64}) shapes.push_back(PlanShape{rows, 0, 0, 2});
        // the plans are built on host threads at once (host tables read only;
        // each thread makes its own uploads), then timed one by one
        int dev = 0;
        RTG_CUDA(cudaGetDevice(&dev));
        std::vector<std::future<ApplyPlan*>> built;
        for (const PlanShape& sh : shapes)
            built.push_back(std::async(std::launch::async, [h, sh, par, dev]() {
                RTG_CUDA(cudaSetDevice(dev));
                return shape_plan<T>(h, sh, par);
            }));
        std::vector<ApplyPlan*> plans(shapes.size(), nullptr);
        std::exception_ptr failed;
        for (size_t q = 0; q < built.size(); ++q) {
            try {
                plans[q] = built[q].get();
            } catch (...) {
                if (!failed) failed = std::current_exception();
            }
        }
        if (failed) {
            for (ApplyPlan* p : plans) free_plan(p);
            std::rethrow_exception(failed);
        }
        for (size_t q = 0; q < shapes.size(); ++q) {
            const PlanShape& sh = shapes[q];
            ApplyPlan* p = plans[q];
            plans[q] = nullptr;
            TuneRecord r{sh, 0, -1, p->ntiles, p->tg_begin[kSmemClasses], plan_launches(p)};
            float tt = 1e30f;
            try {
                tt = time_plan<T>(h, p, x, y, e0, e1, s);
            } catch (...) {
                free_plan(p);
                for (ApplyPlan* rest : plans) free_plan(rest);
                throw;
            }
            r.ns = (int)std::min(tt * 1e6f, 2.e9f);
            recs.push_back(r);
            if (tt < tbest) {
                free_plan(best);
                best = p;
                tbest = tt;
                ibest = (int)recs.size() - 1;
            } else {
                free_plan(p);
            }
        }
    } catch (...) {
        free_plan(best);
        if (par) free_parity(par);
        release();
        throw;
    }
    release();
    recs[ibest].chosen = 1;
    best->own_par = f64;
    best->tuning = std::move(recs);
    return best;
}

// Replaces the apply plan of one precision by the plan of a given shape.
template <typename T>
static void force_shape(rtg_handle* h, const PlanShape& sh) {
    constexpr bool f64 = sizeof(T) == 8;
    ParityTables* par = f64 ? build_parity(h) : nullptr;
    ApplyPlan* p = nullptr;
    try {
        p = shape_plan<T>(h, sh, par);
    } catch (...) {
        if (par) free_parity(par);
        throw;
    }
    p->own_par = f64;
    p->tuning.push_back(TuneRecord{sh, 1, -1, p->ntiles, p->tg_begin[kSmemClasses], plan_launches(p)});
    set_plan_attributes<T>(p);
    ApplyPlan*& slot = f64 ? h->plan64 : h->plan32;
    free_plan(slot);
    slot = p;
}

int apply_shape(rtg_handle* h, int prec, const int32_t* shape) {
    if (!shape) {   // back to the autotuned plan on the next apply
        ApplyPlan*& slot = prec == RTG_FP64 ? h->plan64 : h->plan32;
        free_plan(slot);
        slot = nullptr;
        return 0;
    }
    const PlanShape sh{shape[0], shape[1], shape[2], shape[3]};
    if (sh.rows < 1 || sh.rows > 1024 || sh.gcap < 0 || (sh.split != 0 && sh.split != 1) ||
        sh.tc < 0 || sh.tc > 2 || (prec == RTG_FP64 && sh.tc))
        throw RtgError{RTG_ERR_ARG, "apply shape: rows in [1, 1024], gcap >= 0, split 0 or 1, tc 0, 1 or 2 (tc: FP32 only)"};
    if (prec == RTG_FP64)
        force_shape<double>(h, sh);
    else
        force_shape<float>(h, sh);
    return 0;
}

int apply_tuning(rtg_handle* h, int32_t* out, int cap_rows, cudaStream_t s) {
    if (!h->plan32) {
        h->plan32 = tune_plan<float>(h, s);
        set_plan_attributes<float>(h->plan32);
    }
    const auto& rec = h->plan32->tuning;
    const int n = (int)rec.size();
    for (int i = 0; i < std::min(n, cap_rows); ++i) {
        int32_t* o = out + (size_t)i * 9;
        o[0] = rec[i].shape.rows;
        o[1] = rec[i].shape.gcap;
        o[2] = rec[i].shape.split;
        o[3] = rec[i].shape.tc;
        o[4] = rec[i].chosen;
        o[5] = rec[i].ns;
        o[6] = rec[i].items;
        o[7] = rec[i].groups;
        o[8] = rec[i].launches;
    }
    return n;
}

int apply_status(rtg_handle* h, cudaStream_t s) {
    const ApplyPlan* p = h->plan32;
    if (h->poisoned) return RTG_ERR_TIMEOUT;
    if (!p || !p->ntc) return RTG_OK;
    int st = 0;
    RTG_CUDA(cudaMemcpyAsync(&st, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    RTG_CUDA(cudaStreamSynchronize(s));
    if (st) h->poisoned = true;
    return st ? RTG_ERR_TIMEOUT : RTG_OK;
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
    if (h->poisoned)
        throw RtgError{RTG_ERR_TIMEOUT, "a tensor-core wait of this handle timed out earlier; destroy the handle"};
    constexpr bool f64 = sizeof(T) == 8;
    ApplyPlan*& plan = f64 ? h->plan64 : h->plan32;
    if (!plan) {
        plan = tune_plan<T>(h, s);
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

// Error indicators and hp steering of the AMR loop, on the device: the step
// after the solve (src/amr/Error_Indicator).
//   * angular jump (error/error_angular_jump.py:14-98): per element the
//     squared jump of u between the cell's top and bottom (theta pull-back +1
//     and -1) and its angular neighbours' bottom and top, integrated over the
//     column's LGL nodes; per column the sum over its cells;
//   * spatial jump (error/error_spatial_jump.py:17-247): per column the
//     squared jump of the face traces against every neighbour column's
//     facing traces, both projected onto the finer face interval's LGL rule
//     (the larger node count) times the smaller angular cell's LG rule,
//     divided by perimeter * 2 pi;
//   * hp steering (col_hp_steer.py:14-64, cell_hp_steer.py:15-48): the
//     Legendre-decay estimate lp of the angle-integrated solution per column
//     and of the space-integrated solution per cell.
// Set-up (once per handle, on the host): angular neighbours of every element
// (the cells of a column partition [0, 2 pi), ordered by theta), the pairs
// (element, facing neighbour element) of the spatial jump with their
// interpolation matrices, and node tables.  Kernels are one CTA per element
// or column with fixed-order sums.
#include <algorithm>
#include <cmath>
#include <map>
#include <unordered_map>
#include <vector>

#include "rtg_internal.h"

namespace rtg {

namespace {

constexpr int kNT = kMaxNodes * (kMaxNodes + 1);   // one node table [n][i]
constexpr double kTwoPiD = 6.283185307179586;      // 2 * numpy.pi

// One (self element, neighbour element) pair of the spatial jump.  Matrix
// offsets index the pair table: psi [n0 x nB], psi1 [n1 x nB] (face-direction
// Lagrange bases at the common rule's nodes), xsi0 [nth0 x nH], xsi1
// [nth1 x nH] (angular), wB [nB], wH [nH].
struct JumpPair {
    int32_t e0, e1, face, n0, n1, nB, nth0, nth1, nH;
    int32_t psi0, psi1, xsi0, xsi1, wB, wH, pad;
    double coef;   // dA * dth_G / 4
};

// Table layout (doubles): LGL nodes, LGL weights, LG nodes, LG weights, LG
// basis at +1, LG basis at -1 (each [kMaxNodes+1][kMaxNodes]); Legendre
// values P_k at the LGL and at the LG nodes ([kMaxNodes+1][k][i], each
// kMaxNodes * kNT); then the pair matrices.
enum { kLglX = 0, kLglW = 1, kLgX = 2, kLgW = 3, kLgTop = 4, kLgBot = 5, kNodeTables = 6 };
constexpr size_t kLegLgl = (size_t)kNodeTables * kNT;
constexpr size_t kLegLg = kLegLgl + (size_t)kMaxNodes * kNT;
constexpr size_t kTabHead = kLegLg + (size_t)kMaxNodes * kNT;

// P_k at node i of the n-node LGL (lg = false) or LG (lg = true) rule
__device__ __forceinline__ double leg_at(const double* tab, bool lg, int n, int k, int i) {
    return tab[(lg ? kLegLg : kLegLgl) + (size_t)n * kMaxNodes * kMaxNodes + (size_t)k * kMaxNodes + i];
}

__device__ __forceinline__ const double* ntab(const double* tab, int which, int n) {
    return tab + (size_t)which * kNT + (size_t)n * kMaxNodes;
}

// top/bot[enode_off[e] + ij] = sum_a u[e, ij, a] l_a(+1 / -1)
__global__ void ang_trace_kernel(OpView<double> v, const double* __restrict__ tab, const double* __restrict__ u,
                                 const int64_t* __restrict__ enode_off, double* __restrict__ top,
                                 double* __restrict__ bot) {
    const int e = blockIdx.x;
    const ElemDev E = v.elems[e];
    const ColDev C = v.cols[E.col];
    const int nn = C.nx * C.ny, nth = E.nth;
    const double* lt = ntab(tab, kLgTop, nth);
    const double* lb = ntab(tab, kLgBot, nth);
    for (int ij = threadIdx.x; ij < nn; ij += blockDim.x) {
        const double* ue = u + E.dof_off + (int64_t)ij * nth;
        double st = 0., sb = 0.;
        for (int a = 0; a < nth; ++a) {
            st += ue[a] * lt[a];
            sb += ue[a] * lb[a];
        }
        top[enode_off[e] + ij] = st;
        bot[enode_off[e] + ij] = sb;
    }
}

// cell_err2[e] = 1/4 sum_ij wx_i wy_j 0.5 ((bot_e - top_lower)^2 + (top_e - bot_upper)^2)
__global__ void ang_jump_kernel(OpView<double> v, const double* __restrict__ tab, const int32_t* __restrict__ cnbr,
                                const int64_t* __restrict__ enode_off, const double* __restrict__ top,
                                const double* __restrict__ bot, double* __restrict__ cell_err2) {
    __shared__ double red[256];
    const int e = blockIdx.x;
    const ElemDev E = v.elems[e];
    const ColDev C = v.cols[E.col];
    const int nn = C.nx * C.ny;
    const int lo = cnbr[2 * e], up = cnbr[2 * e + 1];
    const double* wx = ntab(tab, kLglW, C.nx);
    const double* wy = ntab(tab, kLglW, C.ny);
    double acc = 0.;
    for (int ij = threadIdx.x; ij < nn; ij += blockDim.x) {
        const double jl = bot[enode_off[e] + ij] - top[enode_off[lo] + ij];
        const double ju = top[enode_off[e] + ij] - bot[enode_off[up] + ij];
        acc += wx[ij / C.ny] * wy[ij % C.ny] * 0.5 * (jl * jl + ju * ju);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) cell_err2[e] = 0.25 * red[0];
}

// col_err2[c] = sum of its cells' values, cells in order
__global__ void col_sum_kernel(OpView<double> v, const double* __restrict__ cell_val, double* __restrict__ col_val) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= v.ncols) return;
    const ColDev C = v.cols[c];
    double s = 0.;
    for (int e = C.elem_begin; e < C.elem_end; ++e) s += cell_val[e];
    col_val[c] = s;
}

// node index (i*ny + j) of the q-th node of face F of an nx x ny grid
__device__ __forceinline__ int face_node(int F, int q, int nx, int ny) {
    switch (F) {
        case 0: return (nx - 1) * ny + q;   // i = nx-1, j = q
        case 1: return q * ny + ny - 1;     // i = q, j = ny-1
        case 2: return q;                   // i = 0, j = q
        default: return q * ny;             // i = q, j = 0
    }
}

constexpr int kJumpWarps = 8;

// One CTA per column, one warp per pair: both traces projected onto the
// common rule (angular contraction first, then along the face), the weighted
// squared difference summed with a fixed shuffle tree; the column sums its
// pairs in order: col_err2 = sum / (perimeter * 2 pi).
__global__ void __launch_bounds__(32 * kJumpWarps)
spt_jump_kernel(OpView<double> v, const double* __restrict__ tab, const JumpPair* __restrict__ pairs,
                const int32_t* __restrict__ pstart, const double* __restrict__ u, double* __restrict__ pairval,
                double* __restrict__ col_err2) {
    __shared__ double T0[kJumpWarps][kMaxNodes * kMaxNodes];
    __shared__ double T1[kJumpWarps][kMaxNodes * kMaxNodes];
    const int c = blockIdx.x;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p0 = pstart[c], p1 = pstart[c + 1];
    for (int p = p0 + w; p < p1; p += kJumpWarps) {
        const JumpPair P = pairs[p];
        const ElemDev E0 = v.elems[P.e0], E1 = v.elems[P.e1];
        const ColDev C0 = v.cols[E0.col], C1 = v.cols[E1.col];
        const int F1 = (P.face + 2) % 4;   // the neighbour's facing face
        const double* xsi0 = tab + P.xsi0;
        const double* xsi1 = tab + P.xsi1;
        for (int t = lane; t < P.n0 * P.nH; t += 32) {
            const int j = t / P.nH, ap = t % P.nH;
            const double* ue = u + E0.dof_off + (int64_t)face_node(P.face, j, C0.nx, C0.ny) * P.nth0;
            double s = 0.;
            for (int a = 0; a < P.nth0; ++a) s += ue[a] * xsi0[a * P.nH + ap];
            T0[w][t] = s;
        }
        for (int t = lane; t < P.n1 * P.nH; t += 32) {
            const int q = t / P.nH, ap = t % P.nH;
            const double* ue = u + E1.dof_off + (int64_t)face_node(F1, q, C1.nx, C1.ny) * P.nth1;
            double s = 0.;
            for (int a = 0; a < P.nth1; ++a) s += ue[a] * xsi1[a * P.nH + ap];
            T1[w][t] = s;
        }
        __syncwarp();
        const double* psi0 = tab + P.psi0;
        const double* psi1 = tab + P.psi1;
        const double* wB = tab + P.wB;
        const double* wH = tab + P.wH;
        double acc = 0.;
        for (int t = lane; t < P.nB * P.nH; t += 32) {
            const int jp = t / P.nH, ap = t % P.nH;
            double a0 = 0., a1 = 0.;
            for (int j = 0; j < P.n0; ++j) a0 += psi0[j * P.nB + jp] * T0[w][j * P.nH + ap];
            for (int q = 0; q < P.n1; ++q) a1 += psi1[q * P.nB + jp] * T1[w][q * P.nH + ap];
            const double d = a0 - a1;
            acc += wB[jp] * wH[ap] * d * d;
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) pairval[p] = P.coef * acc;
        __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.;
        for (int p = p0; p < p1; ++p) s += __ldcg(pairval + p);
        const ColDev C = v.cols[c];
        col_err2[c] = s / ((2. * C.dx + 2. * C.dy) * kTwoPiD);
    }
}

// Per column: uh[i][j] = sum_cells (dth/2) sum_a wth_a u, W = wx wy uh, then
// a_nx,j = (2nx-1)(2j+1)/4 sum_i sum_q P_{nx-1}(x_i) W[i][q] P_j(y_q) and its
// transpose counterpart (contracted one index at a time), and
// lp = (term_x + term_y) / 2.
__global__ void hp_col_kernel(OpView<double> v, const double* __restrict__ tab, const double* __restrict__ u,
                              double* __restrict__ col_lp) {
    __shared__ double W[kMaxNodes * kMaxNodes];
    __shared__ double rx[kMaxNodes], ry[kMaxNodes], ax[kMaxNodes], ay[kMaxNodes];
    const int c = blockIdx.x;
    const ColDev C = v.cols[c];
    const int nx = C.nx, ny = C.ny, nn = nx * ny;
    const double* wx = ntab(tab, kLglW, nx);
    const double* wy = ntab(tab, kLglW, ny);
    for (int ij = threadIdx.x; ij < nn; ij += blockDim.x) {
        double uh = 0.;
        for (int e = C.elem_begin; e < C.elem_end; ++e) {
            const ElemDev E = v.elems[e];
            const double* wt = ntab(tab, kLgW, E.nth);
            const double* ue = u + E.dof_off + (int64_t)ij * E.nth;
            double s = 0.;
            for (int a = 0; a < E.nth; ++a) s += wt[a] * ue[a];
            uh += (E.dth / 2.) * s;
        }
        W[ij] = wx[ij / ny] * wy[ij % ny] * uh;
    }
    __syncthreads();
    // rx[q] = sum_i P_{nx-1}(x_i) W[i][q]; ry[i] = sum_q W[i][q] P_{ny-1}(y_q)
    if ((int)threadIdx.x < ny) {
        const int q = threadIdx.x;
        double s = 0.;
        for (int i = 0; i < nx; ++i) s += leg_at(tab, false, nx, nx - 1, i) * W[i * ny + q];
        rx[q] = s;
    } else if ((int)threadIdx.x >= 32 && (int)threadIdx.x < 32 + nx) {
        const int i = threadIdx.x - 32;
        double s = 0.;
        for (int q = 0; q < ny; ++q) s += W[i * ny + q] * leg_at(tab, false, ny, ny - 1, q);
        ry[i] = s;
    }
    __syncthreads();
    if ((int)threadIdx.x < ny) {
        const int j = threadIdx.x;
        double s = 0.;
        for (int q = 0; q < ny; ++q) s += rx[q] * leg_at(tab, false, ny, j, q);
        ax[j] = (2. * nx - 1.) * (2. * j + 1.) / 4. * s;
    } else if ((int)threadIdx.x >= 32 && (int)threadIdx.x < 32 + nx) {
        const int i = threadIdx.x - 32;
        double s = 0.;
        for (int p = 0; p < nx; ++p) s += leg_at(tab, false, nx, i, p) * ry[p];
        ay[i] = (2. * i + 1.) * (2. * ny - 1.) / 4. * s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sx = 0., sy = 0.;
        for (int j = 0; j < ny; ++j) sx += ax[j] * ax[j] * (2. / (2. * j + 1.));
        for (int i = 0; i < nx; ++i) sy += ay[i] * ay[i] * (2. / (2. * i + 1.));
        const double t0 = log((2. * nx - 1.) / (2. * sx)) / (2. * log(nx - 1.));
        const double t1 = log((2. * ny - 1.) / (2. * sy)) / (2. * log(ny - 1.));
        col_lp[c] = 0.5 * (t0 + t1);
    }
}

// Per element (one warp): uh[a] = (dx dy / 4) sum_ij wx wy u, then
// a = (2 nth - 1)/2 sum_a wth_a uh_a P_{nth-1}(th_a) and
// lp = log((2 nth - 1) / (2 a^2 2/(2 nth - 1))) / (2 log(nth - 1)).
__global__ void hp_cell_kernel(OpView<double> v, const double* __restrict__ tab, const double* __restrict__ u,
                               double* __restrict__ cell_lp) {
    const int lane = threadIdx.x & 31;
    const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (e >= v.nelem) return;
    const ElemDev E = v.elems[e];
    const ColDev C = v.cols[E.col];
    const int nth = E.nth, nn = C.nx * C.ny;
    const double* wx = ntab(tab, kLglW, C.nx);
    const double* wy = ntab(tab, kLglW, C.ny);
    const double* wt = ntab(tab, kLgW, nth);
    // lanes over (node, angle) pairs: coalesced reads of the element
    double part = 0.;
    for (int t = lane; t < nn * nth; t += 32) {
        const int ij = t / nth, a = t % nth;
        part += wx[ij / C.ny] * wy[ij % C.ny] * u[E.dof_off + t] * wt[a] * leg_at(tab, true, nth, nth - 1, a);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if (lane == 0) {
        const double an = (2. * nth - 1.) / 2. * ((C.dx * C.dy) / 4. * part);
        const double asq = an * an * (2. / (2. * nth - 1.));
        cell_lp[e] = log((2. * nth - 1.) / (2. * asq)) / (2. * log((double)nth - 1.));
    }
}

// i-th Lagrange basis of `nodes` at x, zero outside [-1-1e-14, 1+1e-14]
// (dg/quadrature/lag_eval.py:3-19)
double lagrange(const double* nodes, int n, int i, double x) {
    if (!((-1.0 - 1.e-14 <= x) && (x <= 1.0 + 1.e-14))) return 0.;
    double r = 1.;
    for (int j = 0; j < n; ++j)
        if (j != i) r *= (x - nodes[j]) / (nodes[i] - nodes[j]);
    return r;
}

double push_fw(double x0, double x1, double s) { return x0 + (x1 - x0) / 2.0 * (s + 1.0); }
double pull_bk(double x0, double x1, double x) { return -1.0 + 2.0 / (x1 - x0) * (x - x0); }

int64_t key_of(int lv, int idx) {
    int64_t base = 0;
    for (int l = 0; l < lv; ++l) base += (int64_t)1 << l;
    return base + idx;
}

}  // namespace

struct AmrTables {
    std::vector<void*> allocs;
    double* d_tab = nullptr;
    int32_t* d_cnbr = nullptr;
    int64_t* d_enode_off = nullptr;
    double *d_top = nullptr, *d_bot = nullptr;
    JumpPair* d_pairs = nullptr;
    int32_t* d_pstart = nullptr;
    double* d_pairval = nullptr;
    int64_t npairs = 0;
};

namespace {

template <typename T>
T* amr_upload(AmrTables* a, const std::vector<T>& v) {
    void* p = nullptr;
    RTG_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(v.size(), 1)));
    a->allocs.push_back(p);
    if (!v.empty()) RTG_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return (T*)p;
}

AmrTables* get_amr(rtg_handle* h) {
    if (h->amr) return h->amr;
    const HostTables& t = h->host;
    const int nc = (int)t.cols.size(), ne = (int)t.elems.size();
    AmrTables* a = new AmrTables();
    try {
        // node tables
        std::vector<double> tab((size_t)kNodeTables * kNT, 0.);
        tab.reserve(kTabHead);
        double xw[2][kMaxNodes];
        for (int n = 1; n <= kMaxNodes; ++n) {
            quad_lgl(n, xw[0], xw[1]);
            for (int i = 0; i < n; ++i) {
                tab[(size_t)kLglX * kNT + n * kMaxNodes + i] = xw[0][i];
                tab[(size_t)kLglW * kNT + n * kMaxNodes + i] = xw[1][i];
            }
            quad_lg(n, xw[0], xw[1]);
            for (int i = 0; i < n; ++i) {
                tab[(size_t)kLgX * kNT + n * kMaxNodes + i] = xw[0][i];
                tab[(size_t)kLgW * kNT + n * kMaxNodes + i] = xw[1][i];
                tab[(size_t)kLgTop * kNT + n * kMaxNodes + i] = lagrange(xw[0], n, i, 1.);
                tab[(size_t)kLgBot * kNT + n * kMaxNodes + i] = lagrange(xw[0], n, i, -1.);
            }
        }
        tab.resize(kTabHead, 0.);
        for (int lgrule = 0; lgrule < 2; ++lgrule)
            for (int n = 1; n <= kMaxNodes; ++n) {
                const double* xs = &tab[(size_t)(lgrule ? kLgX : kLglX) * kNT + (size_t)n * kMaxNodes];
                for (int i = 0; i < n; ++i) {
                    // P_k(x) by the three-term recurrence
                    double p0 = 1., p1 = xs[i];
                    for (int k = 0; k < kMaxNodes; ++k) {
                        const double pk = k == 0 ? 1. : (k == 1 ? xs[i] : 0.);
                        double val = pk;
                        if (k >= 2) {
                            const double p2 = ((2. * (k - 1) + 1.) * xs[i] * p1 - (k - 1) * p0) / k;
                            p0 = p1;
                            p1 = p2;
                            val = p2;
                        }
                        tab[(lgrule ? kLegLg : kLegLgl) + (size_t)n * kMaxNodes * kMaxNodes + (size_t)k * kMaxNodes + i] =
                            val;
                    }
                }
            }
        auto nodes = [&](int which, int n) { return &tab[(size_t)which * kNT + (size_t)n * kMaxNodes]; };
        // angular neighbours: the column's cells in theta order, cyclic
        std::vector<int32_t> cnbr(2 * (size_t)ne, 0);
        std::vector<int64_t> enode_off(ne + 1, 0);
        for (int c = 0; c < nc; ++c) {
            const ColDev& C = t.cols[c];
            std::vector<int> ord;
            for (int e = C.elem_begin; e < C.elem_end; ++e) ord.push_back(e);
            std::sort(ord.begin(), ord.end(), [&](int x, int y) { return t.cell_pos[2 * x] < t.cell_pos[2 * y]; });
            const int k = (int)ord.size();
            for (int q = 0; q < k; ++q) {
                cnbr[2 * ord[q]] = ord[(q + k - 1) % k];
                cnbr[2 * ord[q] + 1] = ord[(q + 1) % k];
            }
            for (int e = C.elem_begin; e < C.elem_end; ++e) enode_off[e + 1] = enode_off[e] + C.nx * C.ny;
        }
        // spatial-jump pairs (error/error_spatial_jump.py:33-233), in the
        // reference's loop order: face, neighbour column, own cell, neighbour cell
        std::vector<std::unordered_map<int64_t, int32_t>> key2elem(nc);
        for (int c = 0; c < nc; ++c)
            for (int e = t.cols[c].elem_begin; e < t.cols[c].elem_end; ++e)
                key2elem[c][key_of(t.cell_lv[e], t.cell_idx[e])] = e;
        std::map<std::vector<double>, int32_t> seen;
        auto put = [&](const std::vector<double>& m) {
            auto f = seen.find(m);
            if (f != seen.end()) return f->second;
            const int32_t off = (int32_t)tab.size();
            tab.insert(tab.end(), m.begin(), m.end());
            seen.emplace(m, off);
            return off;
        };
        std::vector<JumpPair> pairs;
        std::vector<int32_t> pstart(nc + 1, 0);
        for (int c0 = 0; c0 < nc; ++c0) {
            const ColDev& C0 = t.cols[c0];
            const double* q0 = &t.col_pos[4 * (size_t)c0];
            for (int F = 0; F < 4; ++F) {
                const int k1 = t.col_nbr_raw[8 * (size_t)c0 + 2 * F], k2 = t.col_nbr_raw[8 * (size_t)c0 + 2 * F + 1];
                int nbrs[2] = {-1, -1}, nnb = 0;
                if (k1 >= 0) nbrs[nnb++] = k1;
                if (k2 >= 0 && k2 != k1) nbrs[nnb++] = k2;
                for (int s = 0; s < nnb; ++s) {
                    const int c1 = nbrs[s];
                    const ColDev& C1 = t.cols[c1];
                    const double* q1 = &t.col_pos[4 * (size_t)c1];
                    const bool alongy = F % 2 == 0;
                    const double a0 = alongy ? q0[1] : q0[0], b0 = alongy ? q0[3] : q0[2];
                    const double a1 = alongy ? q1[1] : q1[0], b1 = alongy ? q1[3] : q1[2];
                    const double d0 = b0 - a0, d1 = b1 - a1;
                    const double aA = d0 <= d1 ? a0 : a1, bA = d0 <= d1 ? b0 : b1, dA = d0 <= d1 ? d0 : d1;
                    const int n0 = alongy ? C0.ny : C0.nx, n1 = alongy ? C1.ny : C1.nx;
                    const int nB = std::max(n0, n1);
                    const double* sB = nodes(kLglX, nB);
                    std::vector<double> psi0((size_t)n0 * nB), psi1((size_t)n1 * nB), wB(nodes(kLglW, nB), nodes(kLglW, nB) + nB);
                    for (int jp = 0; jp < nB; ++jp) {
                        const double xf = push_fw(aA, bA, sB[jp]);
                        const double s0 = pull_bk(a0, b0, xf), s1 = pull_bk(a1, b1, xf);
                        for (int j = 0; j < n0; ++j) psi0[(size_t)j * nB + jp] = lagrange(nodes(kLglX, n0), n0, j, s0);
                        for (int q = 0; q < n1; ++q) psi1[(size_t)q * nB + jp] = lagrange(nodes(kLglX, n1), n1, q, s1);
                    }
                    const int32_t opsi0 = put(psi0), opsi1 = put(psi1), owB = put(wB);
                    for (int e0 = C0.elem_begin; e0 < C0.elem_end; ++e0) {
                        // neighbour cells (dg/mesh/nhbr_cells_in_nhbr_col.py:14-65)
                        int nbc[2] = {-1, -1};
                        const auto& km = key2elem[c1];
                        const int clv = t.cell_lv[e0], cidx = t.cell_idx[e0];
                        auto fs = km.find(key_of(clv, cidx));
                        if (fs != km.end()) {
                            nbc[0] = fs->second;
                        } else {
                            const int64_t kp = (clv - 1 >= 0) ? key_of(clv - 1, cidx / 2) : (int64_t)(cidx / 2);
                            auto fp = km.find(kp);
                            if (fp != km.end()) nbc[0] = fp->second;
                            auto f0 = km.find(key_of(clv + 1, 2 * cidx));
                            if (f0 != km.end()) {
                                nbc[0] = f0->second;
                                auto f1 = km.find(key_of(clv + 1, 2 * cidx + 1));
                                if (f1 != km.end()) nbc[1] = f1->second;
                            }
                        }
                        const ElemDev& E0 = t.elems[e0];
                        const double t00 = t.cell_pos[2 * e0], t01 = t.cell_pos[2 * e0 + 1];
                        for (int q = 0; q < 2; ++q) {
                            const int e1 = nbc[q];
                            if (e1 < 0) continue;
                            const ElemDev& E1 = t.elems[e1];
                            const double t10 = t.cell_pos[2 * e1], t11 = t.cell_pos[2 * e1 + 1];
                            const double dt0 = t01 - t00, dt1 = t11 - t10;
                            const double gA = dt0 <= dt1 ? t00 : t10, gB = dt0 <= dt1 ? t01 : t11;
                            const double dG = dt0 <= dt1 ? dt0 : dt1;
                            const int nH = std::max(E0.nth, E1.nth);
                            const double* sH = nodes(kLgX, nH);
                            std::vector<double> xsi0((size_t)E0.nth * nH), xsi1((size_t)E1.nth * nH);
                            std::vector<double> wH(nodes(kLgW, nH), nodes(kLgW, nH) + nH);
                            for (int ap = 0; ap < nH; ++ap) {
                                const double th = push_fw(gA, gB, sH[ap]);
                                const double s0 = pull_bk(t00, t01, th), s1 = pull_bk(t10, t11, th);
                                for (int aa = 0; aa < E0.nth; ++aa)
                                    xsi0[(size_t)aa * nH + ap] = lagrange(nodes(kLgX, E0.nth), E0.nth, aa, s0);
                                for (int rr = 0; rr < E1.nth; ++rr)
                                    xsi1[(size_t)rr * nH + ap] = lagrange(nodes(kLgX, E1.nth), E1.nth, rr, s1);
                            }
                            JumpPair P{};
                            P.e0 = e0;
                            P.e1 = e1;
                            P.face = F;
                            P.n0 = n0;
                            P.n1 = n1;
                            P.nB = nB;
                            P.nth0 = E0.nth;
                            P.nth1 = E1.nth;
                            P.nH = nH;
                            P.psi0 = opsi0;
                            P.psi1 = opsi1;
                            P.xsi0 = put(xsi0);
                            P.xsi1 = put(xsi1);
                            P.wB = owB;
                            P.wH = put(wH);
                            P.coef = dA * dG / 4.;
                            pairs.push_back(P);
                        }
                    }
                }
            }
            pstart[c0 + 1] = (int32_t)pairs.size();
        }
        if (tab.size() > (size_t)INT32_MAX) throw RtgError{RTG_ERR_SIZE, "error-indicator tables too large"};
        a->npairs = (int64_t)pairs.size();
        a->d_tab = amr_upload(a, tab);
        a->d_cnbr = amr_upload(a, cnbr);
        a->d_enode_off = amr_upload(a, enode_off);
        a->d_pairs = amr_upload(a, pairs);
        a->d_pstart = amr_upload(a, pstart);
        std::vector<double> zero_nodes((size_t)enode_off[ne], 0.), zero_pairs(pairs.size(), 0.);
        a->d_top = amr_upload(a, zero_nodes);
        a->d_bot = amr_upload(a, zero_nodes);
        a->d_pairval = amr_upload(a, zero_pairs);
    } catch (...) {
        for (void* p : a->allocs) cudaFree(p);
        delete a;
        throw;
    }
    h->amr = a;
    return a;
}

}  // namespace

void free_amr(rtg_handle* h) {
    if (!h->amr) return;
    for (void* p : h->amr->allocs) cudaFree(p);
    delete h->amr;
    h->amr = nullptr;
}

void error_angular_jump(rtg_handle* h, const double* u, double* cell_err2, double* col_err2, cudaStream_t s) {
    AmrTables* a = get_amr(h);
    const OpView<double>& v = h->v64;
    ang_trace_kernel<<<v.nelem, 128, 0, s>>>(v, a->d_tab, u, a->d_enode_off, a->d_top, a->d_bot), count_launch();
    ang_jump_kernel<<<v.nelem, 256, 0, s>>>(v, a->d_tab, a->d_cnbr, a->d_enode_off, a->d_top, a->d_bot, cell_err2),
        count_launch();
    if (col_err2) col_sum_kernel<<<(v.ncols + 127) / 128, 128, 0, s>>>(v, cell_err2, col_err2), count_launch();
    RTG_LAUNCHED("error_angular_jump kernels");
}

void error_spatial_jump(rtg_handle* h, const double* u, double* col_err2, cudaStream_t s) {
    AmrTables* a = get_amr(h);
    const OpView<double>& v = h->v64;
    spt_jump_kernel<<<v.ncols, 32 * kJumpWarps, 0, s>>>(v, a->d_tab, a->d_pairs, a->d_pstart, u, a->d_pairval,
                                                       col_err2), count_launch();
    RTG_LAUNCHED("spt_jump_kernel");
}

void hp_steer(rtg_handle* h, const double* u, double* col_lp, double* cell_lp, cudaStream_t s) {
    AmrTables* a = get_amr(h);
    const OpView<double>& v = h->v64;
    if (col_lp) hp_col_kernel<<<v.ncols, 64, 0, s>>>(v, a->d_tab, u, col_lp), count_launch();
    if (cell_lp) hp_cell_kernel<<<(v.nelem + 7) / 8, 256, 0, s>>>(v, a->d_tab, u, cell_lp), count_launch();
    RTG_LAUNCHED("hp steering kernels");
}

int64_t error_jump_pairs(rtg_handle* h) { return get_amr(h)->npairs; }

}  // namespace rtg

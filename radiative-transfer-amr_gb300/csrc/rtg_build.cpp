// Host-side construction of the matrix-free operator tables from a flattened
// hp mesh: quadrature rules, Lagrange derivative tables, spatial and angular
// mortar matrices, face couplings and the per-column angular scattering
// matrices.  Each formula cites the reference routine it restates.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <unordered_map>

#include "rtg_internal.h"

namespace rtg {

static const double kPi = 3.141592653589793;  // numpy.pi / consts.PI

// ------------------------------------------------------------- quadrature
// Legendre-Gauss-Lobatto rule (dg/quadrature/lgl_quad.py:3-40): Newton on
// x P_N(x) - P_{N-1}(x) from Chebyshev-Lobatto points with the reference's
// step divisor (n + 1), stop when the update is <= 2.3e-16; flipped to
// ascending order (dg/quadrature/quad_xyth.py:43-45).
void quad_lgl(int n, double* x, double* w) {
    if (n == 1) {
        x[0] = 0.;
        w[0] = 2.;
        return;
    }
    std::vector<double> xs(n), xo(n), P((size_t)n * n);
    for (int k = 0; k < n; ++k) xs[k] = std::cos(kPi * k / (n - 1));
    for (int k = 0; k < n; ++k) xo[k] = xs[k] + 1.;
    for (int it = 0; it < 10000; ++it) {
        double dmax = 0.;
        for (int k = 0; k < n; ++k) dmax = std::max(dmax, std::fabs(xs[k] - xo[k]));
        if (!(dmax > 2.3e-16)) break;
        for (int m = 0; m < n; ++m) {
            double* p = &P[(size_t)m * n];
            p[0] = 1.;
            p[1] = xs[m];
            for (int k = 1; k < n - 1; ++k)
                p[k + 1] = ((2 * k + 1) * xs[m] * p[k] - k * p[k - 1]) / (k + 1);
        }
        for (int m = 0; m < n; ++m) {
            const double* p = &P[(size_t)m * n];
            xo[m] = xs[m];
            xs[m] = xo[m] - (xo[m] * p[n - 1] - p[n - 2]) / ((n + 1) * p[n - 1]);
        }
    }
    for (int m = 0; m < n; ++m) {
        const double pn = P[(size_t)m * n + n - 1];
        x[n - 1 - m] = xs[m];
        w[n - 1 - m] = 2. / ((n - 1) * n * pn * pn);
    }
}

// Legendre-Gauss rule (dg/quadrature/lg_quad.py:3-49): Newton on L_n from the
// shifted Chebyshev guess, derivative with the (n + 1) factor and the weights'
// ((n+1)/n)^2 correction, flipped to ascending (quad_xyth.py:79-81).
void quad_lg(int n, double* x, double* w) {
    if (n == 1) {
        x[0] = 0.;
        w[0] = 2.;
        return;
    }
    std::vector<double> y(n), yo(n), Lp(n), L((size_t)n * (n + 1));
    for (int k = 0; k < n; ++k) {
        const double xu = (k == n - 1) ? 1.0 : (-1.0 + k * (2.0 / (n - 1)));
        y[k] = std::cos((2 * k + 1) * kPi / (2 * n)) +
               (0.27 / n) * std::sin(kPi * xu * (n - 1) / (n + 1));
    }
    for (int k = 0; k < n; ++k) yo[k] = y[k] + 1.;
    for (int m = 0; m < n; ++m) L[(size_t)m * (n + 1)] = 1.;
    for (int it = 0; it < 10000; ++it) {
        double dmax = 0.;
        for (int k = 0; k < n; ++k) dmax = std::max(dmax, std::fabs(y[k] - yo[k]));
        if (!(dmax > 2.3e-16)) break;
        for (int m = 0; m < n; ++m) {
            double* l = &L[(size_t)m * (n + 1)];
            l[1] = y[m];
            for (int k = 1; k < n; ++k) l[k + 1] = ((2 * k + 1) * y[m] * l[k] - k * l[k - 1]) / (k + 1);
            Lp[m] = (n + 1) * (l[n - 1] - y[m] * l[n]) / (1 - y[m] * y[m]);
        }
        for (int m = 0; m < n; ++m) {
            yo[m] = y[m];
            y[m] = yo[m] - L[(size_t)m * (n + 1) + n] / Lp[m];
        }
    }
    const double c = (double)(n + 1) / n;
    for (int m = 0; m < n; ++m) {
        const double node = (-1. * (1 - y[m]) + 1. * (1 + y[m])) / 2;
        x[n - 1 - m] = node;
        w[n - 1 - m] = c * c * 2. / ((1 - y[m] * y[m]) * Lp[m] * Lp[m]);
    }
}

namespace {

struct Rule {
    double x[kMaxNodes], w[kMaxNodes];
};

const Rule& lgl(int n) {
    static Rule cache[kMaxNodes + 1];
    static bool done[kMaxNodes + 1] = {false};
    if (!done[n]) {
        quad_lgl(n, cache[n].x, cache[n].w);
        done[n] = true;
    }
    return cache[n];
}

const Rule& lg(int n) {
    static Rule cache[kMaxNodes + 1];
    static bool done[kMaxNodes + 1] = {false};
    if (!done[n]) {
        quad_lg(n, cache[n].x, cache[n].w);
        done[n] = true;
    }
    return cache[n];
}

// i-th Lagrange basis of `nodes` at x, zero outside the reference interval
// widened by 1e-14 (dg/quadrature/lag_eval.py:3-19).
double lag(const double* nodes, int n, int i, double x) {
    if (!((-1.0 - 1.e-14 <= x) && (x <= 1.0 + 1.e-14))) return 0.;
    double r = 1.;
    for (int j = 0; j < n; ++j)
        if (j != i) r *= (x - nodes[j]) / (nodes[i] - nodes[j]);
    return r;
}

// Exact derivative of the j-th Lagrange basis (dg/quadrature/lag_ddx.py:44-62).
double lag_d(const double* nodes, int n, int j, double x) {
    double r = 0.;
    for (int k = 0; k < n; ++k) {
        if (k == j) continue;
        double p = 1.;
        for (int i = 0; i < n; ++i)
            if (i != j && i != k) p *= (x - nodes[i]) / (nodes[j] - nodes[i]);
        r += p / (nodes[j] - nodes[k]);
    }
    return r;
}

inline double push(double a, double b, double t) { return a + (b - a) / 2.0 * (t + 1.0); }
inline double pull(double a, double b, double x) { return -1.0 + 2.0 / (b - a) * (x - a); }

// Spatial mortar E (n1 x n0, row-major) coupling the facing node line of a
// neighbour column into column 0 (rt/get_Ex.py:10-127 == rt/get_Ey.py:9-125).
void spatial_mortar(int n0, int n1, double a0, double b0, double a1, double b1, int lv0, int lv1,
                    double* E) {
    const Rule& R0 = lgl(n0);
    const Rule& R1 = lgl(n1);
    for (int k = 0; k < n0 * n1; ++k) E[k] = 0.;
    if (lv0 - lv1 == -1) {
        const double c = 1. / 2.;
        if (n0 > n1) {
            double tb[kMaxNodes];
            for (int q = 0; q < n0; ++q) tb[q] = pull(a0, b0, push(a1, b1, R0.x[q]));
            for (int i = 0; i < n1; ++i)
                for (int p = 0; p < n0; ++p)
                    for (int q = 0; q < n0; ++q)
                        E[i * n0 + p] += c * R0.w[q] * lag(R1.x, n1, i, R0.x[q]) * lag(R0.x, n0, p, tb[q]);
        } else {
            for (int i = 0; i < n1; ++i) {
                const double t = pull(a0, b0, push(a1, b1, R1.x[i]));
                for (int p = 0; p < n0; ++p) E[i * n0 + p] = c * R1.w[i] * lag(R0.x, n0, p, t);
            }
        }
    } else {
        if (n0 >= n1) {
            for (int p = 0; p < n0; ++p) {
                const double t = pull(a1, b1, push(a0, b0, R0.x[p]));
                for (int i = 0; i < n1; ++i) E[i * n0 + p] = R0.w[p] * lag(R1.x, n1, i, t);
            }
        } else {
            double tb[kMaxNodes];
            for (int q = 0; q < n1; ++q) tb[q] = pull(a1, b1, push(a0, b0, R1.x[q]));
            for (int i = 0; i < n1; ++i)
                for (int p = 0; p < n0; ++p)
                    for (int q = 0; q < n1; ++q)
                        E[i * n0 + p] += R1.w[q] * lag(R1.x, n1, i, tb[q]) * lag(R0.x, n0, p, R1.x[q]);
        }
    }
}

// Angular mortar E_th (n1 x n0, row-major) for cell [c00, c01] and neighbour
// cell [c10, c11] across face F, with Theta_F = cos(th - F pi/2) and entries
// below 1e-15 zeroed (rt/get_Eth.py:9-154).
void angular_mortar(int n0, int n1, double c00, double c01, double c10, double c11, int lv0,
                    int lv1, int F, double* E) {
    const Rule& R0 = lg(n0);
    const Rule& R1 = lg(n1);
    for (int k = 0; k < n0 * n1; ++k) E[k] = 0.;
    const double sh = F * kPi / 2.;
    if (lv0 - lv1 == -1) {
        if (n0 > n1) {
            double th[kMaxNodes], tb[kMaxNodes], TF[kMaxNodes];
            for (int q = 0; q < n0; ++q) {
                th[q] = push(c10, c11, R0.x[q]);
                TF[q] = std::cos(th[q] - sh);
                tb[q] = pull(c00, c01, th[q]);
            }
            for (int a = 0; a < n1; ++a)
                for (int r = 0; r < n0; ++r)
                    for (int q = 0; q < n0; ++q)
                        E[a * n0 + r] += R0.w[q] * TF[q] * lag(R1.x, n1, a, R0.x[q]) * lag(R0.x, n0, r, tb[q]);
        } else {
            for (int a = 0; a < n1; ++a) {
                const double th = push(c10, c11, R1.x[a]);
                const double TF = std::cos(th - sh);
                const double tb = pull(c00, c01, th);
                for (int r = 0; r < n0; ++r) E[a * n0 + r] = R1.w[a] * TF * lag(R0.x, n0, r, tb);
            }
        }
        for (int k = 0; k < n0 * n1; ++k) E[k] *= 1. / 2.;
    } else {
        if (n0 >= n1) {
            for (int r = 0; r < n0; ++r) {
                const double th = push(c00, c01, R0.x[r]);
                const double TF = std::cos(th - sh);
                const double tb = pull(c10, c11, th);
                for (int a = 0; a < n1; ++a) E[a * n0 + r] = R0.w[r] * TF * lag(R1.x, n1, a, tb);
            }
        } else {
            double TF[kMaxNodes], tb[kMaxNodes];
            for (int q = 0; q < n1; ++q) {
                const double th = push(c00, c01, R1.x[q]);
                TF[q] = std::cos(th - sh);
                tb[q] = pull(c10, c11, th);
            }
            for (int a = 0; a < n1; ++a)
                for (int r = 0; r < n0; ++r)
                    for (int q = 0; q < n1; ++q)
                        E[a * n0 + r] += R1.w[q] * TF[q] * lag(R1.x, n1, a, tb[q]) * lag(R0.x, n0, r, R1.x[q]);
        }
    }
    for (int k = 0; k < n0 * n1; ++k)
        if (std::fabs(E[k]) < 1.e-15) E[k] = 0.0;
}

// Face F is outflow for an angular cell in quadrant q
// (rt/boundary_convection_matrix.py:270-273).
bool is_outflow(int q, int F) {
    return (q == 0 && (F == 0 || F == 1)) || (q == 1 && (F == 1 || F == 2)) ||
           (q == 2 && (F == 2 || F == 3)) || (q == 3 && (F == 3 || F == 0));
}

// Inflow-boundary faces for the interior mask (dg/matrix/get_masks.py:160-190).
bool is_inflow_quadrant(int q, int F) {
    switch (F) {
        case 0: return q == 1 || q == 2;
        case 1: return q == 2 || q == 3;
        case 2: return q == 3 || q == 0;
        default: return q == 0 || q == 1;
    }
}

int64_t cell_key(int lv, int idx) {
    int64_t base = 0;
    for (int l = 0; l < lv; ++l) base += (int64_t)1 << l;
    return base + idx;
}

void fail(const std::string& m) { throw RtgError{RTG_ERR_MESH, m}; }

}  // namespace

void build_tables(const rtg_mesh_desc* m, const rtg_coeffs* c, HostTables& t) {
    if (!m || !c) throw RtgError{RTG_ERR_ARG, "null mesh or coefficient description"};
    if (m->ncols <= 0 || m->nelem <= 0) fail("empty mesh");
    if (!m->col_pos || !m->col_ndofs || !m->col_lv || !m->col_nbr || !m->col_elem_start ||
        !m->cell_pos || !m->cell_ndof || !m->cell_lv || !m->cell_idx || !m->cell_quadrant)
        throw RtgError{RTG_ERR_ARG, "null array in mesh description"};
    if (!c->kappa || !c->sigma || !c->sig_off || !c->phi || !c->col_sig || c->nsig <= 0)
        throw RtgError{RTG_ERR_ARG, "null array in coefficient description"};
    const int nc = m->ncols, ne = m->nelem;
    if (m->col_elem_start[0] != 0 || m->col_elem_start[nc] != ne) fail("col_elem_start does not cover the elements");
    t.col_pos.assign(m->col_pos, m->col_pos + 4 * (size_t)nc);
    t.cell_pos.assign(m->cell_pos, m->cell_pos + 2 * (size_t)ne);
    t.cell_lv.assign(m->cell_lv, m->cell_lv + ne);
    t.cell_idx.assign(m->cell_idx, m->cell_idx + ne);

    // quadrature tables: LGL weights and G[n][p][i] = l'_p(x_i) w_i
    t.lglw.assign((size_t)(kMaxNodes + 1) * kMaxNodes, 0.);
    t.G.clear();
    for (int n = 1; n <= kMaxNodes; ++n) {
        const Rule& R = lgl(n);
        for (int i = 0; i < n; ++i) t.lglw[(size_t)n * kMaxNodes + i] = R.w[i];
    }
    std::vector<int32_t> goff(kMaxNodes + 1, 0);
    for (int n = 1; n <= kMaxNodes; ++n) {
        goff[n] = (int32_t)t.G.size();
        const Rule& R = lgl(n);
        for (int p = 0; p < n; ++p)
            for (int i = 0; i < n; ++i) t.G.push_back(lag_d(R.x, n, p, R.x[i]) * R.w[i]);
    }

    // columns
    t.cols.resize(nc);
    t.elems.resize(ne);
    int64_t dof = 0;
    int32_t node = 0;
    std::vector<std::unordered_map<int64_t, int32_t>> key2elem(nc);
    for (int ci = 0; ci < nc; ++ci) {
        ColDev& C = t.cols[ci];
        const double* p = m->col_pos + 4 * ci;
        C.dx = p[2] - p[0];
        C.dy = p[3] - p[1];
        C.nx = m->col_ndofs[2 * ci];
        C.ny = m->col_ndofs[2 * ci + 1];
        if (C.nx < 1 || C.ny < 1 || C.nx > kMaxNodes || C.ny > kMaxNodes)
            throw RtgError{RTG_ERR_SIZE, "column degree outside [1, 16] nodes"};
        if (!(C.dx > 0. && C.dy > 0.)) fail("column with non-positive extent");
        C.elem_begin = m->col_elem_start[ci];
        C.elem_end = m->col_elem_start[ci + 1];
        if (C.elem_end <= C.elem_begin) fail("column without cells");
        C.node_off = node;
        node += C.nx * C.ny;
        C.dof_off = dof;
        C.sig = c->col_sig[ci];
        if (C.sig < 0 || C.sig >= c->nsig) fail("col_sig out of range");
        int nth_col = 0;
        int64_t prev_key = -1;
        for (int e = C.elem_begin; e < C.elem_end; ++e) {
            const int nth = m->cell_ndof[e];
            if (nth < 1 || nth > kMaxNodes) throw RtgError{RTG_ERR_SIZE, "cell degree outside [1, 16] nodes"};
            const int64_t k = cell_key(m->cell_lv[e], m->cell_idx[e]);
            if (k <= prev_key) fail("cells of a column are not in increasing key order");
            prev_key = k;
            key2elem[ci][k] = e;
            ElemDev& E = t.elems[e];
            E.dof_off = dof;
            E.col = ci;
            E.nth = nth;
            E.row = nth_col;
            E.dth = m->cell_pos[2 * e + 1] - m->cell_pos[2 * e];
            if (!(E.dth > 0.)) fail("cell with non-positive extent");
            nth_col += nth;
            dof += (int64_t)C.nx * C.ny * nth;
        }
        C.nth_col = nth_col;
        C.ndof = C.nx * C.ny * nth_col;
        t.max_col_ndof = std::max(t.max_col_ndof, C.ndof);
        t.max_nth_col = std::max(t.max_nth_col, nth_col);
        for (int f = 0; f < 4; ++f)
            for (int s = 0; s < 2; ++s) {
                const int nb = m->col_nbr[8 * ci + 2 * f + s];
                if (nb < -1 || nb >= nc) fail("neighbour column index out of range");
            }
    }
    t.ndof = dof;
    t.nnodes = node;

    // distinct face-neighbour columns (first-seen order, -1 padded) and the
    // number of faces without a neighbour
    t.col_nbr_raw.assign(m->col_nbr, m->col_nbr + (size_t)8 * nc);
    t.col_nbr8.assign((size_t)8 * nc, -1);
    t.col_free.assign(nc, 0);
    for (int ci = 0; ci < nc; ++ci) {
        int cnt = 0;
        for (int f = 0; f < 4; ++f) {
            const int a = m->col_nbr[8 * ci + 2 * f], b = m->col_nbr[8 * ci + 2 * f + 1];
            if (a < 0 && b < 0) ++t.col_free[ci];
            for (int nb : {a, b}) {
                if (nb < 0) continue;
                bool seen = false;
                for (int q = 0; q < cnt; ++q) seen |= t.col_nbr8[8 * ci + q] == nb;
                if (!seen) t.col_nbr8[8 * ci + cnt++] = nb;
            }
        }
    }

    // coefficients at column nodes: kw = wx wy kappa, sw = wx wy sigma
    t.kw.resize(node);
    t.sw.resize(node);
    for (int ci = 0; ci < nc; ++ci) {
        const ColDev& C = t.cols[ci];
        const Rule& Rx = lgl(C.nx);
        const Rule& Ry = lgl(C.ny);
        for (int i = 0; i < C.nx; ++i)
            for (int j = 0; j < C.ny; ++j) {
                const int k = C.node_off + i * C.ny + j;
                const double ww = Rx.w[i] * Ry.w[j];
                t.kw[k] = ww * c->kappa[k];
                t.sw[k] = ww * c->sigma[k];
                if (!std::isfinite(t.kw[k]) || !std::isfinite(t.sw[k]))
                    throw RtgError{RTG_ERR_NONFINITE, "non-finite kappa or sigma"};
            }
    }

    // per-cell angular tables, deduplicated by (th0, th1, nth)
    std::map<std::tuple<double, double, int>, int32_t> angmap;
    t.ang.clear();
    for (int e = 0; e < ne; ++e) {
        const double th0 = m->cell_pos[2 * e], th1 = m->cell_pos[2 * e + 1];
        const int nth = m->cell_ndof[e];
        auto key = std::make_tuple(th0, th1, nth);
        auto it = angmap.find(key);
        if (it != angmap.end()) {
            t.elems[e].ang = it->second;
            continue;
        }
        const int32_t off = (int32_t)t.ang.size();
        angmap[key] = off;
        t.elems[e].ang = off;
        t.ang.resize(t.ang.size() + 7 * (size_t)nth);
        const Rule& R = lg(nth);
        double* A = &t.ang[off];
        for (int a = 0; a < nth; ++a) {
            const double th = push(th0, th1, R.x[a]);
            A[a] = R.w[a];
            A[nth + a] = R.w[a] * std::sin(th);
            A[2 * nth + a] = R.w[a] * std::cos(th);
            for (int F = 0; F < 4; ++F) A[(3 + F) * nth + a] = std::cos(th - F * kPi / 2.);
        }
    }

    // angular scattering matrices per signature:
    // W[(K r),(K' a)] = dth_K (dth_K'/2) wth_r wth'_a Phi(th_r, th'_a)
    // (the angular factor of rt/scattering_matrix.py:201-203)
    std::vector<int32_t> sig_col(c->nsig, -1);
    for (int ci = 0; ci < nc; ++ci)
        if (sig_col[t.cols[ci].sig] < 0) sig_col[t.cols[ci].sig] = ci;
    t.W_off.assign(c->nsig + 1, 0);
    t.sig_nth.assign(c->nsig, 0);
    for (int s = 0; s < c->nsig; ++s) {
        const int ci = sig_col[s];
        int nthc = 0;
        if (ci >= 0) nthc = t.cols[ci].nth_col;
        t.sig_nth[s] = nthc;
        if ((int64_t)nthc * nthc != c->sig_off[s + 1] - c->sig_off[s] && ci >= 0)
            fail("Phi block size does not match the column angular mesh");
        t.W_off[s + 1] = t.W_off[s] + (int64_t)nthc * nthc;
    }
    t.W.assign(t.W_off[c->nsig], 0.);
    for (int s = 0; s < c->nsig; ++s) {
        const int ci = sig_col[s];
        if (ci < 0) continue;
        const ColDev& C = t.cols[ci];
        const int nthc = C.nth_col;
        const double* Phi = c->phi + c->sig_off[s];
        double* W = &t.W[t.W_off[s]];
        for (int e0 = C.elem_begin; e0 < C.elem_end; ++e0) {
            const ElemDev& E0 = t.elems[e0];
            const Rule& R0 = lg(E0.nth);
            for (int e1 = C.elem_begin; e1 < C.elem_end; ++e1) {
                const ElemDev& E1 = t.elems[e1];
                const Rule& R1 = lg(E1.nth);
                for (int r = 0; r < E0.nth; ++r)
                    for (int a = 0; a < E1.nth; ++a) {
                        const int64_t k = (int64_t)(E0.row + r) * nthc + (E1.row + a);
                        const double ph = Phi[k];
                        if (!std::isfinite(ph)) throw RtgError{RTG_ERR_NONFINITE, "non-finite Phi"};
                        W[k] = E0.dth * (E1.dth / 2.0) * R0.w[r] * R1.w[a] * ph;
                    }
            }
        }
    }
    // every column of a signature must share the cell structure of its first column
    for (int ci = 0; ci < nc; ++ci) {
        const ColDev& C = t.cols[ci];
        const ColDev& C0 = t.cols[sig_col[C.sig]];
        if (C.nth_col != C0.nth_col || C.elem_end - C.elem_begin != C0.elem_end - C0.elem_begin)
            fail("columns sharing a Phi block have different angular meshes");
        for (int k = 0; k < C.elem_end - C.elem_begin; ++k) {
            const int e = C.elem_begin + k, e0 = C0.elem_begin + k;
            if (m->cell_ndof[e] != m->cell_ndof[e0] || m->cell_pos[2 * e] != m->cell_pos[2 * e0] ||
                m->cell_pos[2 * e + 1] != m->cell_pos[2 * e0 + 1])
                fail("columns sharing a Phi block have different angular meshes");
        }
    }

    // face terms (rt/boundary_convection_matrix.py:160-537)
    t.mort.clear();
    t.cpls.clear();
    std::map<std::tuple<int, int, int, int, int>, int32_t> es_cache;  // dir, n0, n1, dlv, side
    std::map<std::tuple<double, double, double, double, int, int, int, int, int>, int32_t> et_cache;
    t.ndof_interior = 0;
    for (int ci = 0; ci < nc; ++ci) {
        const ColDev& C = t.cols[ci];
        const double* p0 = m->col_pos + 4 * ci;
        const int lv0 = m->col_lv[ci];
        for (int e = C.elem_begin; e < C.elem_end; ++e) {
            ElemDev& E = t.elems[e];
            const int quad = m->cell_quadrant[e];
            const int clv = m->cell_lv[e], cidx = m->cell_idx[e];
            E.flags = 0;
            E.cpl_begin = (int32_t)t.cpls.size();
            for (int F = 0; F < 4; ++F) {
                const int nk1 = m->col_nbr[8 * ci + 2 * F], nk2 = m->col_nbr[8 * ci + 2 * F + 1];
                if (nk1 < 0 && nk2 < 0 && is_inflow_quadrant(quad, F)) E.flags |= 1 << (4 + F);
                if (is_outflow(quad, F)) {
                    E.flags |= 1 << F;
                    continue;
                }
                const double dcoeff = (F % 2 == 0) ? C.dy * E.dth / 4. : C.dx * E.dth / 4.;
                int nbrs[2] = {-1, -1};
                int nn = 0;
                if (nk1 >= 0) nbrs[nn++] = nk1;
                if (nk2 != nk1 && nk2 >= 0) nbrs[nn++] = nk2;
                for (int s = 0; s < nn; ++s) {
                    const int cj = nbrs[s];
                    const ColDev& C1 = t.cols[cj];
                    const double* p1 = m->col_pos + 4 * cj;
                    const int lv1 = m->col_lv[cj];
                    const int dlv = lv0 - lv1;
                    if (dlv < -1 || dlv > 1) fail("spatial neighbours differ by more than one level");
                    // spatial mortar along the face (E_y on x-faces, E_x on y-faces)
                    const int dir = F % 2;  // 0: along y, 1: along x
                    const double a0 = dir == 0 ? p0[1] : p0[0], b0 = dir == 0 ? p0[3] : p0[2];
                    const double a1 = dir == 0 ? p1[1] : p1[0], b1 = dir == 0 ? p1[3] : p1[2];
                    const int n0 = dir == 0 ? C.ny : C.nx, n1 = dir == 0 ? C1.ny : C1.nx;
                    const double mid0 = (a0 + b0) / 2., mid1 = (a1 + b1) / 2.;
                    int side = 0;  // same level
                    if (dlv == -1) side = (mid1 < mid0) ? 1 : 2;
                    if (dlv == 1) side = (mid1 < mid0) ? 2 : 1;
                    auto ek = std::make_tuple(dir, n0, n1, dlv, side);
                    int32_t es;
                    auto eit = es_cache.find(ek);
                    if (eit == es_cache.end()) {
                        es = (int32_t)t.mort.size();
                        t.mort.resize(t.mort.size() + (size_t)n0 * n1);
                        spatial_mortar(n0, n1, a0, b0, a1, b1, lv0, lv1, &t.mort[es]);
                        es_cache[ek] = es;
                    } else {
                        es = eit->second;
                    }
                    // neighbour cells (dg/mesh/nhbr_cells_in_nhbr_col.py:14-65)
                    int nbc[2] = {-1, -1};
                    const auto& km = key2elem[cj];
                    const int64_t k_same = cell_key(clv, cidx);
                    auto f_same = km.find(k_same);
                    if (f_same != km.end()) {
                        nbc[0] = f_same->second;
                    } else {
                        const int64_t kp = (clv - 1 >= 0) ? cell_key(clv - 1, (int)(cidx / 2)) : (int64_t)(cidx / 2);
                        auto fp = km.find(kp);
                        if (fp != km.end()) nbc[0] = fp->second;
                        auto f0 = km.find(cell_key(clv + 1, 2 * cidx));
                        if (f0 != km.end()) {
                            nbc[0] = f0->second;
                            auto f1 = km.find(cell_key(clv + 1, 2 * cidx + 1));
                            if (f1 != km.end()) nbc[1] = f1->second;
                        }
                    }
                    for (int q = 0; q < 2; ++q) {
                        const int e1 = nbc[q];
                        if (e1 < 0) continue;
                        const ElemDev& E1 = t.elems[e1];
                        const double c00 = m->cell_pos[2 * e], c01 = m->cell_pos[2 * e + 1];
                        const double c10 = m->cell_pos[2 * e1], c11 = m->cell_pos[2 * e1 + 1];
                        const int l1 = m->cell_lv[e1];
                        if (clv - l1 < -1 || clv - l1 > 1) fail("angular neighbours differ by more than one level");
                        auto tk = std::make_tuple(c00, c01, c10, c11, E.nth, E1.nth, clv, l1, F);
                        int32_t et;
                        auto tit = et_cache.find(tk);
                        if (tit == et_cache.end()) {
                            et = (int32_t)t.mort.size();
                            t.mort.resize(t.mort.size() + (size_t)E.nth * E1.nth);
                            angular_mortar(E.nth, E1.nth, c00, c01, c10, c11, clv, l1, F, &t.mort[et]);
                            et_cache[tk] = et;
                        } else {
                            et = tit->second;
                        }
                        CplDev cp;
                        cp.dcoeff = dcoeff;
                        cp.face = F;
                        cp.nbr = e1;
                        cp.es = es;
                        cp.et = et;
                        t.cpls.push_back(cp);
                    }
                }
            }
            E.cpl_end = (int32_t)t.cpls.size();
            // unknowns of this element
            const int bm = E.flags >> 4;
            int64_t nb = 0;
            for (int i = 0; i < C.nx; ++i)
                for (int j = 0; j < C.ny; ++j) {
                    const bool bdry = ((bm & 1) && i == C.nx - 1) || ((bm & 2) && j == C.ny - 1) ||
                                      ((bm & 4) && i == 0) || ((bm & 8) && j == 0);
                    if (bdry) nb += E.nth;
                }
            t.ndof_interior += (int64_t)C.nx * C.ny * E.nth - nb;
        }
    }
    (void)goff;
    // per-element, per-column and per-coupling constants in the kernels' own precision
    t.econst.assign(4 * (size_t)ne, 0.);
    for (int e = 0; e < ne; ++e) {
        const ElemDev& E = t.elems[e];
        const ColDev& C = t.cols[E.col];
        t.econst[4 * e + 0] = C.dx * C.dy * E.dth / 8.;
        t.econst[4 * e + 1] = C.dx * E.dth / 4.;
        t.econst[4 * e + 2] = C.dy * E.dth / 4.;
    }
    t.colc.resize(nc);
    for (int ci = 0; ci < nc; ++ci) {
        t.colc[ci] = t.cols[ci].dx * t.cols[ci].dy / 8.;
        t.max_cells_col = std::max(t.max_cells_col, t.cols[ci].elem_end - t.cols[ci].elem_begin);
    }
    t.cplc.resize(t.cpls.size());
    t.cgeo.resize(t.cpls.size());
    for (size_t k = 0; k < t.cpls.size(); ++k) {
        const CplDev& cp = t.cpls[k];
        t.cplc[k] = cp.dcoeff;
        const ElemDev& E1 = t.elems[cp.nbr];
        const ColDev& C1 = t.cols[E1.col];
        CplGeo g{};
        g.nth1 = E1.nth;
        if (cp.face % 2 == 0) {   // x-faces: neighbour's facing column of nodes, along y
            g.base = E1.dof_off + (int64_t)((cp.face == 0) ? 0 : C1.nx - 1) * C1.ny * E1.nth;
            g.stride = E1.nth;
            g.m1 = C1.ny;
        } else {                  // y-faces: neighbour's facing row of nodes, along x
            g.base = E1.dof_off + (int64_t)((cp.face == 1) ? 0 : C1.ny - 1) * E1.nth;
            g.stride = C1.ny * E1.nth;
            g.m1 = C1.nx;
        }
        t.cgeo[k] = g;
    }
}

}  // namespace rtg

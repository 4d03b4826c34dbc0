"""CPU oracle for the steady monochromatic RT solve -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy/scipy, the algorithm of the reference's
``src/rt`` path (jasonltorchinsky/radiative-transfer-amr): the DG system blocks
mass M, scattering S, interior convection IC, boundary convection BC, the
(M - S) block, the forcing and inflow vectors, the inflow-boundary mask, and
the split solve of rt/solve.py:81-101.  It is the checker for the CUDA
library: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may import it, and never as the thing that is measured or
shipped.  It is pinned against golden fixtures that the reference itself
produced (tests/golden/make_golden.py).

It consumes any mesh object with the reference's attributes (``cols`` dict of
columns with ``pos, lv, ndofs, cells, nhbr_keys``; cells with ``pos, idx, lv,
key, ndofs, quadrant``).  Global DOF order: sorted column keys, then sorted
cell keys, then beta = nth*ny*i + nth*j + a (dg/matrix/get_idxs.py:11-24,42-80).
"""

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PI = math.pi
EPS = float(np.finfo(np.float64).resolution)  # consts/__init__.py:11 (1e-15)
SMALL = 1.e1 * EPS                            # rt/scattering_matrix.py:114
BC_TOL = 1.e-15                               # rt/boundary_convection_matrix.py:165

# ------------------------------------------------------------------ quadrature
_LGL = {}
_LG = {}


def lgl_nodes(n):
    """Legendre-Gauss-Lobatto nodes/weights on [-1, 1], ascending
    (dg/quadrature/lgl_quad.py:3-40 with the flip of quad_xyth.py:43-45).
    Newton iteration on x P_N - P_{N-1} from Chebyshev-Lobatto points, step
    divided by (n + 1) as the reference does, until the update is <= 2.3e-16."""
    if n in _LGL:
        return _LGL[n]
    if n < 1:
        raise ValueError("nnodes < 1")
    if n == 1:
        out = (np.asarray([0.]), np.asarray([2.]))
    else:
        x = np.cos(np.pi * np.arange(0, n) / (n - 1))
        P = np.zeros([n, n])
        x_old = x + 1.
        while np.amax(np.abs(x - x_old)) > 2.3e-16:
            P[:, 0] = 1
            P[:, 1] = x
            for k in range(1, n - 1):
                P[:, k + 1] = ((2 * k + 1) * x * P[:, k] - k * P[:, k - 1]) / (k + 1)
            x_old = x.copy()
            x = x_old - (x * P[:, n - 1] - P[:, n - 2]) / ((n + 1) * P[:, n - 1])
        w = 2. / ((n - 1) * n * P[:, n - 1] ** 2)
        out = (np.flip(x), np.flip(w))
    _LGL[n] = out
    return out


def lg_nodes(n):
    """Legendre-Gauss nodes/weights on [-1, 1], ascending
    (dg/quadrature/lg_quad.py:3-49, flipped as in quad_xyth.py:79-81)."""
    if n in _LG:
        return _LG[n]
    if n < 1:
        raise ValueError("nnodes < 1")
    if n == 1:
        out = (np.asarray([0.]), np.asarray([2.]))
    else:
        xu = np.linspace(-1, 1, n)
        y = np.cos((2 * np.arange(0, n) + 1) * np.pi / (2 * n)) \
            + (0.27 / n) * np.sin(np.pi * xu * (n - 1) / (n + 1))
        L = np.zeros([n, n + 1])
        L[:, 0] = 1
        y_old = y + 1.
        while np.amax(np.abs(y - y_old)) > 2.3e-16:
            L[:, 1] = y
            for k in range(1, n):
                L[:, k + 1] = ((2 * k + 1) * y * L[:, k] - k * L[:, k - 1]) / (k + 1)
            Lp = (n + 1) * (L[:, n - 1] - y * L[:, n]) / (1 - y ** 2)
            y_old = y.copy()
            y = y_old - L[:, n] / Lp
        w = ((n + 1) / n) ** 2 * 2. / ((1 - y ** 2) * Lp ** 2)
        out = (np.flip(y), np.flip(w))
    _LG[n] = out
    return out


def lag(nodes, i, x):
    """i-th Lagrange basis at x, zero outside [-1-1e-14, 1+1e-14]
    (dg/quadrature/lag_eval.py:3-19)."""
    if not (-1.0 - 1.e-14 <= x <= 1.0 + 1.e-14):
        return 0.
    r = 1.
    for j in range(len(nodes)):
        if j != i:
            r *= (x - nodes[j]) / (nodes[i] - nodes[j])
    return r


def lag_d(nodes, j, x):
    """Exact derivative of the j-th Lagrange basis (dg/quadrature/lag_ddx.py:44-62)."""
    n = len(nodes)
    r = 0.
    for k in range(n):
        if k == j:
            continue
        p = 1.
        for i in range(n):
            if i != j and i != k:
                p *= (x - nodes[i]) / (nodes[j] - nodes[i])
        r += p / (nodes[j] - nodes[k])
    return r


def lag_mat(nodes, xs):
    """B[i, m] = l_i(xs[m])."""
    return np.array([[lag(nodes, i, x) for x in xs] for i in range(len(nodes))])


def push(a, b, t):
    return a + (b - a) / 2.0 * (t + 1.0)          # dg/projection/push_pull.py:10-17


def pull(a, b, x):
    return -1.0 + 2.0 / (b - a) * (x - a)         # dg/projection/push_pull.py:19-26


# -------------------------------------------------------------------- mortars
def spatial_mortar(n0, n1, a0, b0, a1, b1, lv0, lv1):
    """E (n1 x n0) coupling the facing node line of a neighbour column (1) into
    column 0 along one spatial direction (rt/get_Ex.py:10-127 and
    rt/get_Ey.py:9-125, which are the same formula in x and in y)."""
    t0, w0 = lgl_nodes(n0)
    t1, w1 = lgl_nodes(n1)
    E = np.zeros([n1, n0])
    if lv0 - lv1 == -1:                       # neighbour is finer
        c = 1. / 2.
        if n0 > n1:
            A = lag_mat(t1, t0)                               # l^1_i(t0_p')
            B = lag_mat(t0, pull(a0, b0, push(a1, b1, t0)))   # l^0_p(...)
            for i in range(n1):
                for p in range(n0):
                    for q in range(n0):
                        E[i, p] += c * w0[q] * A[i, q] * B[p, q]
        else:
            B = lag_mat(t0, pull(a0, b0, push(a1, b1, t1)))   # l^0_p(t1 mapped)
            for i in range(n1):
                for p in range(n0):
                    E[i, p] = c * w1[i] * B[p, i]
    else:
        if n0 >= n1:
            A = lag_mat(t1, pull(a1, b1, push(a0, b0, t0)))
            for i in range(n1):
                for p in range(n0):
                    E[i, p] = w0[p] * A[i, p]
        else:
            A = lag_mat(t1, pull(a1, b1, push(a0, b0, t1)))
            B = lag_mat(t0, t1)
            for i in range(n1):
                for p in range(n0):
                    for q in range(n1):
                        E[i, p] += w1[q] * A[i, q] * B[p, q]
    return E


def angular_mortar(n0, n1, c0, c1, lv0, lv1, F):
    """E_th (n1 x n0) for cell 0 = [c0] and neighbour cell 1 = [c1] across face F,
    including Theta_F = cos(th - F pi/2) (rt/get_Eth.py:9-154)."""
    t0, w0 = lg_nodes(n0)
    t1, w1 = lg_nodes(n1)
    E = np.zeros([n1, n0])
    if lv0 - lv1 == -1:
        c = 1. / 2.
        if n0 > n1:
            th = push(c1[0], c1[1], t0)
            TF = np.cos(th - F * np.pi / 2.)
            A = lag_mat(t1, t0)
            B = lag_mat(t0, pull(c0[0], c0[1], th))
            for a in range(n1):
                for r in range(n0):
                    for q in range(n0):
                        E[a, r] += w0[q] * TF[q] * A[a, q] * B[r, q]
        else:
            th = push(c1[0], c1[1], t1)
            TF = np.cos(th - F * np.pi / 2.)
            B = lag_mat(t0, pull(c0[0], c0[1], th))
            for a in range(n1):
                for r in range(n0):
                    E[a, r] = w1[a] * TF[a] * B[r, a]
        E *= c
    else:
        if n0 >= n1:
            th = push(c0[0], c0[1], t0)
            TF = np.cos(th - F * np.pi / 2.)
            A = lag_mat(t1, pull(c1[0], c1[1], th))
            for a in range(n1):
                for r in range(n0):
                    E[a, r] = w0[r] * TF[r] * A[a, r]
        else:
            th = push(c0[0], c0[1], t1)
            TF = np.cos(th - F * np.pi / 2.)
            A = lag_mat(t1, pull(c1[0], c1[1], th))
            B = lag_mat(t0, t1)
            for a in range(n1):
                for r in range(n0):
                    for q in range(n1):
                        E[a, r] += w1[q] * TF[q] * A[a, q] * B[r, q]
    E[np.abs(E) < 1.e-15] = 0.0
    return E


# ----------------------------------------------------------------- mesh walk
def _cell_key(idx, lv):
    return (2 ** lv - 1 if lv > 0 else 0) + idx


def nbr_cells(mesh, ck, kk, nck):
    """Leaf cells of column nck overlapping cell kk of column ck
    (dg/mesh/nhbr_cells_in_nhbr_col.py:14-65)."""
    cell = mesh.cols[ck].cells[kk]
    cells = mesh.cols[nck].cells
    out = [None, None]
    if cell.key in cells:
        out[0] = cell.key
        return out
    pk = _cell_key(int(cell.idx / 2), cell.lv - 1)
    if pk in cells:
        out[0] = pk
    k0 = _cell_key(2 * cell.idx, cell.lv + 1)
    k1 = _cell_key(2 * cell.idx + 1, cell.lv + 1)
    if k0 not in cells:
        return out
    out[0] = k0
    if k1 in cells:
        out[1] = k1
    return out


class Layout:
    """Element list and DOF offsets in the reference's global order."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.col_keys = sorted(mesh.cols.keys())
        self.elems = []           # (col_key, cell_key)
        self.off = {}             # (col_key, cell_key) -> first DOF
        n = 0
        for ck in self.col_keys:
            col = mesh.cols[ck]
            nx, ny = col.ndofs[0], col.ndofs[1]
            for kk in sorted(col.cells.keys()):
                self.elems.append((ck, kk))
                self.off[(ck, kk)] = n
                n += nx * ny * col.cells[kk].ndofs[0]
        self.N = n


def _col_geom(col):
    x0, y0, x1, y1 = col.pos
    nx, ny = col.ndofs[0], col.ndofs[1]
    tx, wx = lgl_nodes(nx)
    ty, wy = lgl_nodes(ny)
    return x0, y0, x1, y1, nx, ny, tx, wx, ty, wy


def _field(fn, xx, yy, nx, ny):
    v = np.asarray(fn(xx.reshape([nx, 1]), yy.reshape([1, ny])), dtype=np.float64)
    return np.broadcast_to(v, (nx, ny)).copy()


def _eval_nodes(fn, X, Y, T):
    """Evaluate f(x, y, th) on broadcast node arrays; fall back to a scalar loop
    for callables that only take scalars."""
    try:
        v = np.asarray(fn(X, Y, T), dtype=np.float64)
        return np.broadcast_to(v, np.broadcast(X, Y, T).shape).copy()
    except Exception:
        shp = np.broadcast(X, Y, T).shape
        Xb, Yb, Tb = (np.broadcast_to(a, shp) for a in (X, Y, T))
        out = np.empty(shp)
        for idx in np.ndindex(shp):
            out[idx] = fn(float(Xb[idx]), float(Yb[idx]), float(Tb[idx]))
        return out


def _phi_block(Phi, th0, th1):
    try:
        v = np.asarray(Phi(th0[:, None], th1[None, :]), dtype=np.float64)
        return np.broadcast_to(v, (len(th0), len(th1))).copy()
    except Exception:
        return np.array([[Phi(a, b) for b in th1] for a in th0], dtype=np.float64)


def _coo(rows, cols, vals, N):
    if rows:
        r = np.concatenate(rows)
        c = np.concatenate(cols)
        v = np.concatenate(vals)
    else:
        r = c = np.zeros(0, dtype=np.int64)
        v = np.zeros(0)
    return sp.coo_matrix((v, (r, c)), shape=(N, N)).tocsr()


# ------------------------------------------------------------------ operators
def mass_matrix(mesh, kappa, L=None):
    """Diagonal extinction matrix (rt/mass_matrix.py:108-180)."""
    L = L or Layout(mesh)
    diag = np.zeros(L.N)
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        K = wx.reshape(nx, 1) * wy.reshape(1, ny) * _field(kappa, push(x0, x1, tx), push(y0, y1, ty), nx, ny)
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            _, wth = lg_nodes(nth)
            dc = (x1 - x0) * (y1 - y0) * (cell.pos[1] - cell.pos[0]) / 8.
            v = dc * wth[None, None, :] * K[:, :, None]
            o = L.off[(ck, kk)]
            diag[o:o + nx * ny * nth] = v.reshape(-1)
    return sp.diags(diag, format="csr")


def _scat_blocks(mesh, sigma, Phi, L, kappa=None):
    """(rows, cols, vals) of the dense-in-angle column blocks of the scattering
    matrix (rt/scattering_matrix.py:106-247) or, with ``kappa``, of the
    extinction-minus-scattering block (rt/preconditioner_matrix.py:363-514),
    with the reference's |val| <= 1e-14 drop rule."""
    R, C, V = [], [], []
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        dx, dy = x1 - x0, y1 - y0
        xx, yy = push(x0, x1, tx), push(y0, y1, ty)
        Sw = wx.reshape(nx, 1) * wy.reshape(1, ny) * _field(sigma, xx, yy, nx, ny)
        Kw = None
        if kappa is not None:
            Kw = wx.reshape(nx, 1) * wy.reshape(1, ny) * _field(kappa, xx, yy, nx, ny)
        items = sorted(col.cells.items())
        for k0, c0 in items:
            n0 = c0.ndofs[0]
            tb0, w0 = lg_nodes(n0)
            th0 = push(c0.pos[0], c0.pos[1], tb0)
            dth0 = c0.pos[1] - c0.pos[0]
            dc = dx * dy * dth0 / 8
            o0 = L.off[(ck, k0)]
            for k1, c1 in items:
                n1 = c1.ndofs[0]
                tb1, w1 = lg_nodes(n1)
                th1 = push(c1.pos[0], c1.pos[1], tb1)
                dth1 = c1.pos[1] - c1.pos[0]
                o1 = L.off[(ck, k1)]
                Ph = _phi_block(Phi, th0, th1)
                # val = -dcoeff*(dth1/2)*wx*wy*sigma*w0_r*w1_a*Phi_ra, same operation order
                val = (((-dc * (dth1 / 2.0)) * Sw[:, :, None, None]) * w0[None, None, :, None]) \
                    * w1[None, None, None, :] * Ph[None, None, :, :]
                if k0 != k1:
                    keep = (np.abs(Sw) > SMALL)[:, :, None, None] & (np.abs(val) > SMALL)
                else:
                    if Kw is not None:
                        ext = w1[None, None, :] * Kw[:, :, None]             # r == a
                        scat = (dth1 / 2.0) * Sw[:, :, None, None] * w0[None, None, :, None] \
                            * w1[None, None, None, :] * Ph[None, None, :, :]
                        val = -dc * scat
                        rr = np.arange(n0)
                        val[:, :, rr, rr] = dc * (ext - scat[:, :, rr, rr])
                    keep = np.abs(val) > SMALL
                I, J, Rr, Aa = np.nonzero(keep)
                R.append(o0 + n0 * ny * I + n0 * J + Rr)
                C.append(o1 + n1 * ny * I + n1 * J + Aa)
                V.append(val[I, J, Rr, Aa])
    return R, C, V


def scattering_matrix(mesh, sigma, Phi, L=None):
    L = L or Layout(mesh)
    return _coo(*_scat_blocks(mesh, sigma, Phi, L), L.N)


def preconditioner_matrix(mesh, kappa, sigma, Phi, L=None):
    """M - S in one block (rt/preconditioner_matrix.py:22-114)."""
    L = L or Layout(mesh)
    return _coo(*_scat_blocks(mesh, sigma, Phi, L, kappa=kappa), L.N)


def interior_convection_matrix(mesh, L=None):
    """Volume streaming term (rt/interior_convection_matrix.py:110-250):
    IC[(i,q,a),(i,j,a)] = (dx dth/4) wx_i wy_j wth_a sin(th_a) l'_q(y_j)
    IC[(p,j,a),(i,j,a)] = (dy dth/4) wx_i wy_j wth_a cos(th_a) l'_p(x_i)."""
    L = L or Layout(mesh)
    R, C, V = [], [], []
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        dx, dy = x1 - x0, y1 - y0
        WW = wx.reshape(nx, 1) * wy.reshape(1, ny)
        Dy = np.array([[lag_d(ty, q, ty[j]) for j in range(ny)] for q in range(ny)])  # [q, j]
        Dx = np.array([[lag_d(tx, p, tx[i]) for i in range(nx)] for p in range(nx)])  # [p, i]
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            tb, wth = lg_nodes(nth)
            thf = push(cell.pos[0], cell.pos[1], tb)
            dth = cell.pos[1] - cell.pos[0]
            ws, wc = wth * np.sin(thf), wth * np.cos(thf)
            o = L.off[(ck, kk)]
            # term 1: rows (i, q, a), cols (i, j, a)
            dc = dx * dth / 4.
            v1 = dc * WW[:, :, None, None] * ws[None, None, :, None] * Dy.T[None, :, None, :]
            I, J, A, Q = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nth), np.arange(ny),
                                     indexing="ij")
            R.append(o + nth * ny * I.ravel() + nth * Q.ravel() + A.ravel())
            C.append(o + nth * ny * I.ravel() + nth * J.ravel() + A.ravel())
            V.append(v1.ravel())
            # term 2: rows (p, j, a), cols (i, j, a)
            dc = dy * dth / 4.
            v2 = dc * WW[:, :, None, None] * wc[None, None, :, None] * Dx.T[:, None, None, :]
            I, J, A, P = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nth), np.arange(nx),
                                     indexing="ij")
            R.append(o + nth * ny * P.ravel() + nth * J.ravel() + A.ravel())
            C.append(o + nth * ny * I.ravel() + nth * J.ravel() + A.ravel())
            V.append(v2.ravel())
    return _coo(R, C, V, L.N)


def _is_outflow(quadrant, F):
    """Face F is outflow for an angular cell in this quadrant
    (rt/boundary_convection_matrix.py:270-273)."""
    return ((quadrant == 0 and F in (0, 1)) or (quadrant == 1 and F in (1, 2))
            or (quadrant == 2 and F in (2, 3)) or (quadrant == 3 and F in (3, 0)))


def boundary_convection_matrix(mesh, L=None):
    """Face terms (rt/boundary_convection_matrix.py:160-540): outflow faces add
    a diagonal on the face nodes; other faces couple to the facing node line of
    each neighbour element through E_x/E_y (x) E_th."""
    L = L or Layout(mesh)
    R, C, V = [], [], []
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        dx, dy = x1 - x0, y1 - y0
        for F in range(4):
            nk1, nk2 = col.nhbr_keys[F][0], col.nhbr_keys[F][1]
            nbr_cols = []
            if nk1 is not None:
                nbr_cols.append(nk1)
            if nk2 != nk1 and nk2 is not None:
                nbr_cols.append(nk2)
            for kk in sorted(col.cells.keys()):
                cell = col.cells[kk]
                n0 = cell.ndofs[0]
                dth = cell.pos[1] - cell.pos[0]
                o0 = L.off[(ck, kk)]
                dc = dy * dth / 4. if F % 2 == 0 else dx * dth / 4.
                if _is_outflow(cell.quadrant, F):
                    tb, wth = lg_nodes(n0)
                    TF = np.cos(push(cell.pos[0], cell.pos[1], tb) - F * PI / 2.)
                    if F % 2 == 0:
                        xi = nx - 1 if F == 0 else 0
                        val = dc * wy[:, None] * wth[None, :] * TF[None, :]
                        Jj, Aa = np.nonzero(np.abs(val) > BC_TOL)
                        idx = o0 + n0 * ny * xi + n0 * Jj + Aa
                    else:
                        yi = ny - 1 if F == 1 else 0
                        val = dc * wx[:, None] * wth[None, :] * TF[None, :]
                        Jj, Aa = np.nonzero(np.abs(val) > BC_TOL)
                        idx = o0 + n0 * ny * Jj + n0 * yi + Aa
                    R.append(idx)
                    C.append(idx)
                    V.append(val[Jj, Aa])
                    continue
                for nck in nbr_cols:
                    ncol = mesh.cols[nck]
                    mx, my = ncol.ndofs[0], ncol.ndofs[1]
                    if F % 2 == 0:
                        Es = spatial_mortar(ny, my, y0, y1, ncol.pos[1], ncol.pos[3], col.lv, ncol.lv)
                    else:
                        Es = spatial_mortar(nx, mx, x0, x1, ncol.pos[0], ncol.pos[2], col.lv, ncol.lv)
                    for nkk in nbr_cells(mesh, ck, kk, nck):
                        if nkk is None:
                            continue
                        ncell = ncol.cells[nkk]
                        n1 = ncell.ndofs[0]
                        Et = angular_mortar(n0, n1, cell.pos, ncell.pos, cell.lv, ncell.lv, F)
                        o1 = L.off[(nck, nkk)]
                        # val[j, q, a, r] = dcoeff * Es[j, q] * Et[a, r]
                        val = dc * Es[:, :, None, None] * Et[None, None, :, :]
                        Jj, Qq, Aa, Rr = np.nonzero(np.abs(val) > BC_TOL)
                        if F % 2 == 0:
                            xi0 = nx - 1 if F == 0 else 0
                            xi1 = 0 if F == 0 else mx - 1
                            rows = o0 + n0 * ny * xi0 + n0 * Qq + Rr
                            cols = o1 + n1 * my * xi1 + n1 * Jj + Aa
                        else:
                            yi0 = ny - 1 if F == 1 else 0
                            yi1 = 0 if F == 1 else my - 1
                            rows = o0 + n0 * ny * Qq + n0 * yi0 + Rr
                            cols = o1 + n1 * my * Jj + n1 * yi1 + Aa
                        R.append(rows)
                        C.append(cols)
                        V.append(val[Jj, Qq, Aa, Rr])
    return _coo(R, C, V, L.N)


def interior_mask(mesh, L=None):
    """True for unknowns, False for inflow-boundary face nodes of cells whose
    quadrant points into the domain through a face without neighbour
    (dg/matrix/get_masks.py:22-129)."""
    L = L or Layout(mesh)
    mask = np.ones(L.N, dtype=bool)
    inflow = {0: (1, 2), 1: (2, 3), 2: (3, 0), 3: (0, 1)}
    for ck in L.col_keys:
        col = mesh.cols[ck]
        nx, ny = col.ndofs[0], col.ndofs[1]
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            o = L.off[(ck, kk)]
            m = np.ones([nx, ny, nth], dtype=bool)
            for F in range(4):
                if col.nhbr_keys[F][0] is None and col.nhbr_keys[F][1] is None \
                        and cell.quadrant in inflow[F]:
                    if F == 0:
                        m[nx - 1, :, :] = False
                    elif F == 1:
                        m[:, ny - 1, :] = False
                    elif F == 2:
                        m[0, :, :] = False
                    else:
                        m[:, 0, :] = False
            mask[o:o + nx * ny * nth] = m.reshape(-1)
    return mask


def forcing_vector(mesh, f, L=None):
    """f_beta = (dx dy dth/8) wx_i wy_j wth_a f(x_i, y_j, th_a)
    (rt/forcing_vector.py:103-155)."""
    L = L or Layout(mesh)
    out = np.zeros(L.N)
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        xx, yy = push(x0, x1, tx), push(y0, y1, ty)
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            tb, wth = lg_nodes(nth)
            thf = push(cell.pos[0], cell.pos[1], tb)
            dc = (x1 - x0) * (y1 - y0) * (cell.pos[1] - cell.pos[0]) / 8.
            fv = _eval_nodes(f, xx[:, None, None], yy[None, :, None], thf[None, None, :])
            v = dc * wx[:, None, None] * wy[None, :, None] * wth[None, None, :] * fv
            o = L.off[(ck, kk)]
            out[o:o + nx * ny * nth] = v.reshape(-1)
    return out


def boundary_conditions_vector(mesh, bcs_dirac, L=None):
    """Inflow data sampled at every node (rt/boundary_conditions_vector.py:101-207),
    including the point-source branch for a Dirac in x, y and/or th."""
    L = L or Layout(mesh)
    bcs, dirac = bcs_dirac
    out = np.zeros(L.N)
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        xx, yy = push(x0, x1, tx), push(y0, y1, ty)
        pos = L.off[(ck, sorted(col.cells.keys())[0])]
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            tb, _ = lg_nodes(nth)
            thf = push(cell.pos[0], cell.pos[1], tb)
            # the reference branches on any(dirac), i.e. on truthiness: a
            # Dirac coordinate of 0.0 alone does not select the point-source
            # branch (rt/boundary_conditions_vector.py:142)
            if any(dirac):
                lims = [(x0, x1, tx, xx), (y0, y1, ty, yy), (cell.pos[0], cell.pos[1], tb, thf)]
                inside = [True, True, True]
                fac, crd = [], []
                for d in range(3):
                    a, b, tnod, phys = lims[d]
                    n = len(tnod)
                    if dirac[d] is not None and not (dirac[d] < a or b < dirac[d]):
                        sb = pull(a, b, dirac[d])
                        fac.append(np.array([max(0.0, lag(tnod, m, sb)) for m in range(n)]))
                        crd.append(np.full(n, float(dirac[d])))
                    else:
                        if dirac[d] is not None:
                            inside[d] = False
                        fac.append(np.ones(n))
                        crd.append(phys)
                if any(inside):
                    bv = _eval_nodes(bcs, crd[0][:, None, None], crd[1][None, :, None],
                                     crd[2][None, None, :])
                    v = bv * fac[0][:, None, None] * fac[1][None, :, None] * fac[2][None, None, :]
                    out[pos:pos + nx * ny * nth] = v.reshape(-1)
                    pos += nx * ny * nth
            else:
                bv = _eval_nodes(bcs, xx[:, None, None], yy[None, :, None], thf[None, None, :])
                out[pos:pos + nx * ny * nth] = bv.reshape(-1)
                pos += nx * ny * nth
    return out


# -------------------------------------------------------------------- system
def assemble(mesh, kappa, sigma, Phi, f=None, bcs_dirac=None):
    """All blocks of the reference's solve (rt/solve.py:81-101)."""
    L = Layout(mesh)
    out = {"N": L.N, "layout": L}
    out["M"] = mass_matrix(mesh, kappa, L)
    out["S"] = scattering_matrix(mesh, sigma, Phi, L)
    out["MS"] = preconditioner_matrix(mesh, kappa, sigma, Phi, L)
    out["IC"] = interior_convection_matrix(mesh, L)
    out["BC"] = boundary_convection_matrix(mesh, L)
    out["A"] = ((out["BC"] - out["IC"]) + out["MS"]).tocsr()
    out["mask"] = interior_mask(mesh, L)
    if f is not None:
        out["f"] = forcing_vector(mesh, f, L)
    if bcs_dirac is not None:
        out["g"] = boundary_conditions_vector(mesh, bcs_dirac, L)
    return out


def split_system(A, f, g, mask):
    """A_II, A_IB and rhs = f_I - A_IB g_B (rt/solve.py:85-101)."""
    I = np.nonzero(mask)[0]
    B = np.nonzero(~mask)[0]
    A = A.tocsr()
    A_II = A[I][:, I].tocsc()
    A_IB = A[I][:, B]
    rhs = f[I] - A_IB @ g[B]
    return A_II, A_IB, rhs, I, B


def solve_direct(A, f, g, mask):
    """Direct solve of the split system, merged back with the inflow data
    (rt/solve.py:163 merge_vectors)."""
    A_II, _, rhs, I, B = split_system(A, f, g, mask)
    u = np.zeros(len(mask))
    u[I] = spla.spsolve(A_II, rhs)
    u[B] = g[B]
    return u


def node_coords(mesh, L=None):
    """Physical (x, y, th) of every DOF in global order."""
    L = L or Layout(mesh)
    X = np.zeros(L.N)
    Y = np.zeros(L.N)
    T = np.zeros(L.N)
    for ck in L.col_keys:
        col = mesh.cols[ck]
        x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = _col_geom(col)
        xx, yy = push(x0, x1, tx), push(y0, y1, ty)
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            tb, _ = lg_nodes(nth)
            thf = push(cell.pos[0], cell.pos[1], tb)
            o = L.off[(ck, kk)]
            n = nx * ny * nth
            X[o:o + n] = np.broadcast_to(xx[:, None, None], (nx, ny, nth)).reshape(-1)
            Y[o:o + n] = np.broadcast_to(yy[None, :, None], (nx, ny, nth)).reshape(-1)
            T[o:o + n] = np.broadcast_to(thf[None, None, :], (nx, ny, nth)).reshape(-1)
    return X, Y, T


def l2_weights(mesh, L=None):
    """Quadrature weights (dx dy dth/8) wx wy wth of every DOF: the mass weights
    with kappa = 1 (rt/mass_matrix.py:145-169)."""
    L = L or Layout(mesh)
    return mass_matrix(mesh, lambda x, y: 1.0 + 0. * (x + y), L).diagonal()


def column_block_preconditioner(MS, mask, L):
    """Per-column inverse of the (M - S) block restricted to the unknowns: the
    preconditioner rt/preconditioner_matrix.py:506-507 returns
    (return_preconditioner=True), used here in place of PETSc bjacobi."""
    I = np.nonzero(mask)[0]
    pos = np.full(len(mask), -1, dtype=np.int64)
    pos[I] = np.arange(len(I))
    MS = MS.tocsr()
    blocks = []
    bounds = []
    col_start = [L.off[(ck, sorted(L.mesh.cols[ck].cells.keys())[0])] for ck in L.col_keys] + [L.N]
    for c in range(len(L.col_keys)):
        g = np.arange(col_start[c], col_start[c + 1])
        g = g[mask[g]]
        if len(g) == 0:
            continue
        B = MS[g][:, g].tocsc()
        blocks.append(spla.splu(B))
        bounds.append(pos[g])

    def apply(r):
        z = np.empty_like(r)
        for lu, idx in zip(blocks, bounds):
            z[idx] = lu.solve(r[idx])
        return z

    return spla.LinearOperator((len(I), len(I)), matvec=apply, dtype=np.float64)


def solve_gmres(A, MS, f, g, mask, L, rtol=1e-10, restart=50, maxiter=5000, x0=None):
    """GMRES(restart) on the split system with the per-column (M - S)^-1
    preconditioner; returns (u merged, iterations)."""
    A_II, _, rhs, I, B = split_system(A, f, g, mask)
    P = column_block_preconditioner(MS, mask, L)
    count = [0]

    def cb(_):
        count[0] += 1

    x, info = spla.gmres(A_II.tocsr(), rhs, x0=x0, rtol=rtol, atol=0., restart=restart,
                         maxiter=maxiter, M=P, callback=cb, callback_type="pr_norm")
    u = np.zeros(len(mask))
    u[I] = x
    u[B] = g[B]
    return u, count[0]


# -------------------------------------------------------------------- sweep
def element_of_dof(L):
    """Element index (global order) of every DOF."""
    eid = np.zeros(L.N, dtype=np.int64)
    for e, key in enumerate(L.elems):
        o = L.off[key]
        col = L.mesh.cols[key[0]]
        n = col.ndofs[0] * col.ndofs[1] * col.cells[key[1]].ndofs[0]
        eid[o:o + n] = e
    return eid


def sweep_levels(L, BC):
    """Kahn levels of the graph "element depends on the upwind element it couples
    to" read off the off-element blocks of BC; ready elements are taken lowest
    level first, then lowest index, and a cycle is broken by forcing the
    lowest-index unprocessed element.  This is the order the GPU sweep uses."""
    import heapq
    eid = element_of_dof(L)
    C = BC.tocoo()
    keep = eid[C.row] != eid[C.col]
    pairs = set(zip(eid[C.col][keep].tolist(), eid[C.row][keep].tolist()))   # (upwind, element)
    ne = len(L.elems)
    succ = [[] for _ in range(ne)]
    indeg = np.zeros(ne, dtype=np.int64)
    for p, e in pairs:
        succ[p].append(e)
        indeg[e] += 1
    level = np.full(ne, -1, dtype=np.int64)
    lvl_pred = np.zeros(ne, dtype=np.int64)
    done = np.zeros(ne, dtype=bool)
    heap = [(0, e) for e in range(ne) if indeg[e] == 0]
    heapq.heapify(heap)
    processed, forced = 0, 0
    while processed < ne:
        if not heap:
            while done[forced]:
                forced += 1
            indeg[forced] = 0
            heapq.heappush(heap, (int(lvl_pred[forced]), forced))
        _, e = heapq.heappop(heap)
        if done[e]:
            continue
        done[e] = True
        level[e] = lvl_pred[e]
        processed += 1
        for q in succ[e]:
            if done[q]:
                continue
            lvl_pred[q] = max(lvl_pred[q], level[e] + 1)
            indeg[q] -= 1
            if indeg[q] == 0:
                heapq.heappush(heap, (int(lvl_pred[q]), q))
    return level, eid


class SweepPreconditioner:
    """z = P^{-1} r for the upwind transport sweep: element blocks per angular
    node (extinction, minus interior streaming, plus outflow face terms;
    identity rows at inflow-boundary nodes; no scattering) and the inflow
    couplings to elements on earlier levels."""

    def __init__(self, o, L):
        import scipy.linalg as sla
        self.L = L
        mask = o["mask"]
        BC, IC = o["BC"].tocsr(), o["IC"].tocsr()
        self.level, eid = sweep_levels(L, BC)
        T = (BC - IC).tocsr()
        msd = o["M"].diagonal()
        ne = len(L.elems)
        self.order = sorted(range(ne), key=lambda e: (self.level[e], e))
        self.blocks = []
        self.cpl = []
        for e, key in enumerate(L.elems):
            col = L.mesh.cols[key[0]]
            nx, ny, nth = col.ndofs[0], col.ndofs[1], col.cells[key[1]].ndofs[0]
            o0 = L.off[key]
            n = nx * ny * nth
            sl = np.arange(o0, o0 + n)
            Tee = T[sl][:, sl].toarray()
            facs = []
            for r in range(nth):
                idx = np.arange(nx * ny) * nth + r
                B = Tee[np.ix_(idx, idx)] + np.diag(msd[o0 + idx])
                bd = ~mask[o0 + idx]
                B[bd, :] = 0.
                B[bd, bd] = 1.
                facs.append((idx, sla.lu_factor(B)))
            self.blocks.append((o0, n, facs, mask[sl]))
            # couplings to upwind elements on earlier levels
            rows = T[sl]
            cols_e = eid[rows.indices]
            ups = sorted(set(cols_e.tolist()) - {e})
            cl = []
            for u in ups:
                if self.level[u] < self.level[e]:
                    ku = L.elems[u]
                    cu = L.mesh.cols[ku[0]]
                    ou = L.off[ku]
                    nu = cu.ndofs[0] * cu.ndofs[1] * cu.cells[ku[1]].ndofs[0]
                    cl.append((ou, nu, BC[sl][:, ou:ou + nu].tocsr()))
            self.cpl.append(cl)

    def __call__(self, r):
        import scipy.linalg as sla
        z = np.zeros_like(r)
        for e in self.order:
            o0, n, facs, m = self.blocks[e]
            rhs = np.where(m, r[o0:o0 + n], 0.)
            for ou, nu, Bk in self.cpl[e]:
                rhs -= np.where(m, Bk @ z[ou:ou + nu], 0.)
            ze = np.zeros(n)
            for idx, lu in facs:
                ze[idx] = sla.lu_solve(lu, rhs[idx])
            z[o0:o0 + n] = ze
        return z


def solve_sweep_gmres(o, L, rtol=1e-10, restart=50, maxiter=200):
    """Split system solved by scipy GMRES(restart) with the sweep as
    preconditioner -- the GPU plain method's algorithm on the CPU."""
    A_II, _, rhs, I, B = split_system(o["A"], o["f"], o["g"], o["mask"])
    P = SweepPreconditioner(o, L)
    N = len(o["mask"])

    def pre(v):
        full = np.zeros(N)
        full[I] = v
        return P(full)[I]

    M = spla.LinearOperator(A_II.shape, matvec=pre, dtype=np.float64)
    cnt = [0]
    x, info = spla.gmres(A_II.tocsr(), rhs, rtol=rtol, atol=0., restart=restart, maxiter=maxiter,
                         M=M, callback=lambda _: cnt.__setitem__(0, cnt[0] + 1), callback_type="pr_norm")
    u = np.zeros(N)
    u[I] = x
    u[B] = o["g"][B]
    return u, cnt[0], info

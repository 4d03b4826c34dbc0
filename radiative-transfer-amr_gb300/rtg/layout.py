"""Flatten an hp mesh into the plain arrays of ``rtg_mesh_desc`` and sample the
problem coefficients at the quadrature nodes (``rtg_coeffs``).

Works with any mesh object carrying the reference's attributes
(dg/mesh/class_Mesh.py, column/class_Column.py, column/cell/class_Cell.py).
Global order: sorted column keys, sorted cell keys, beta = nth*ny*i + nth*j + a
(dg/matrix/get_idxs.py:11-80)."""

import ctypes as C
from functools import lru_cache

import numpy as np

from . import _lib


@lru_cache(maxsize=None)
def quad(kind, n):
    """kind 0: LGL (x, y), 1: LG (th); ascending nodes and weights on [-1, 1],
    computed by the library (dg/quadrature/quad_xyth.py:22-86)."""
    lib = _lib.load()
    x = np.zeros(n)
    w = np.zeros(n)
    _lib.check(lib.rtg_quad_nodes(kind, n, _lib.ptr(x, C.c_double), _lib.ptr(w, C.c_double)))
    x.setflags(write=False)
    w.setflags(write=False)
    return x, w


def push(a, b, t):
    return a + (b - a) / 2.0 * (t + 1.0)


def _eval(fn, *args):
    """Evaluate a coefficient callable on broadcast arrays; callables written
    for scalars (as the reference calls them) are evaluated point by point."""
    shp = np.broadcast(*args).shape
    try:
        v = np.asarray(fn(*args), dtype=np.float64)
        return np.broadcast_to(v, shp)
    except Exception:
        vec = np.vectorize(lambda *a: float(fn(*a)), otypes=[np.float64])
        return vec(*args)


class MeshLayout:
    """Flattened mesh + bookkeeping needed to move between the mesh objects and
    the library's vectors."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.col_keys = sorted(mesh.cols.keys())
        cidx = {k: i for i, k in enumerate(self.col_keys)}
        nc = len(self.col_keys)
        self.ncols = nc
        self.col_pos = np.zeros((nc, 4))
        self.col_ndofs = np.zeros((nc, 2), dtype=np.int32)
        self.col_lv = np.zeros(nc, dtype=np.int32)
        self.col_nbr = np.full((nc, 4, 2), -1, dtype=np.int32)
        self.col_elem_start = np.zeros(nc + 1, dtype=np.int32)
        cell_pos, cell_ndof, cell_lv, cell_idx, cell_quad, elem_keys = [], [], [], [], [], []
        for ci, ck in enumerate(self.col_keys):
            col = mesh.cols[ck]
            if not col.is_lf:
                raise ValueError("column {} is not a leaf".format(ck))
            self.col_pos[ci] = col.pos
            self.col_ndofs[ci] = col.ndofs[0:2]
            self.col_lv[ci] = col.lv
            for F in range(4):
                for s in range(2):
                    nk = col.nhbr_keys[F][s]
                    if nk is not None:
                        if nk not in cidx:
                            raise ValueError("column {} names missing neighbour {}".format(ck, nk))
                        self.col_nbr[ci, F, s] = cidx[nk]
            self.col_elem_start[ci] = len(cell_pos)
            for kk in sorted(col.cells.keys()):
                cell = col.cells[kk]
                if not cell.is_lf:
                    raise ValueError("cell {} of column {} is not a leaf".format(kk, ck))
                cell_pos.append(cell.pos)
                cell_ndof.append(cell.ndofs[0])
                cell_lv.append(cell.lv)
                cell_idx.append(cell.idx)
                cell_quad.append(-1 if cell.quadrant is None else cell.quadrant)
                elem_keys.append((ck, kk))
        self.col_elem_start[nc] = len(cell_pos)
        self.nelem = len(cell_pos)
        self.cell_pos = np.asarray(cell_pos, dtype=np.float64).reshape(-1, 2)
        self.cell_ndof = np.asarray(cell_ndof, dtype=np.int32)
        self.cell_lv = np.asarray(cell_lv, dtype=np.int32)
        self.cell_idx = np.asarray(cell_idx, dtype=np.int32)
        self.cell_quadrant = np.asarray(cell_quad, dtype=np.int32)
        self.elem_keys = elem_keys
        nxny = self.col_ndofs[:, 0].astype(np.int64) * self.col_ndofs[:, 1]
        elem_col = np.repeat(np.arange(nc), np.diff(self.col_elem_start))
        self.elem_col = elem_col
        self.elem_ndof = nxny[elem_col] * self.cell_ndof
        self.elem_off = np.zeros(self.nelem + 1, dtype=np.int64)
        np.cumsum(self.elem_ndof, out=self.elem_off[1:])
        self.N = int(self.elem_off[-1])
        self.node_off = np.zeros(nc + 1, dtype=np.int64)
        np.cumsum(nxny, out=self.node_off[1:])

    # ------------------------------------------------------------ descriptors
    def mesh_desc(self):
        keep = [self.col_pos, self.col_ndofs, self.col_lv, self.col_nbr, self.col_elem_start,
                self.cell_pos, self.cell_ndof, self.cell_lv, self.cell_idx, self.cell_quadrant]
        keep = [np.ascontiguousarray(a) for a in keep]
        d = _lib.MeshDesc()
        d.ncols = self.ncols
        d.nelem = self.nelem
        d.col_pos = _lib.ptr(keep[0], C.c_double)
        d.col_ndofs = _lib.ptr(keep[1], C.c_int32)
        d.col_lv = _lib.ptr(keep[2], C.c_int32)
        d.col_nbr = _lib.ptr(keep[3], C.c_int32)
        d.col_elem_start = _lib.ptr(keep[4], C.c_int32)
        d.cell_pos = _lib.ptr(keep[5], C.c_double)
        d.cell_ndof = _lib.ptr(keep[6], C.c_int32)
        d.cell_lv = _lib.ptr(keep[7], C.c_int32)
        d.cell_idx = _lib.ptr(keep[8], C.c_int32)
        d.cell_quadrant = _lib.ptr(keep[9], C.c_int32)
        return d, keep

    # ------------------------------------------------------------ coordinates
    def col_nodes(self, ci):
        x0, y0, x1, y1 = self.col_pos[ci]
        nx, ny = int(self.col_ndofs[ci, 0]), int(self.col_ndofs[ci, 1])
        return push(x0, x1, quad(0, nx)[0]), push(y0, y1, quad(0, ny)[0])

    def cell_nodes(self, e):
        th0, th1 = self.cell_pos[e]
        return push(th0, th1, quad(1, int(self.cell_ndof[e]))[0])

    def sample_spatial(self, fn):
        """fn(x, y) at every column node, called like the reference does with
        x of shape [nx, 1] and y of shape [1, ny] (rt/mass_matrix.py:130-137);
        columns of equal degree are evaluated together."""
        out = np.zeros(int(self.node_off[-1]))
        groups = {}
        for ci in range(self.ncols):
            groups.setdefault((int(self.col_ndofs[ci, 0]), int(self.col_ndofs[ci, 1])), []).append(ci)
        for (nx, ny), cis in groups.items():
            cis = np.asarray(cis)
            xb, yb = quad(0, nx)[0], quad(0, ny)[0]
            X = push(self.col_pos[cis, 0][:, None], self.col_pos[cis, 2][:, None], xb[None, :])
            Y = push(self.col_pos[cis, 1][:, None], self.col_pos[cis, 3][:, None], yb[None, :])
            v = np.asarray(_eval(fn, X[:, :, None], Y[:, None, :]))
            v = np.broadcast_to(v, (len(cis), nx, ny)).reshape(len(cis), nx * ny)
            idx = self.node_off[cis][:, None] + np.arange(nx * ny)[None, :]
            out[idx] = v
        return out

    def node_coords(self):
        """(x, y, th) of every DOF in global order (beta = nth ny i + nth j + a
        within an element), computed once per layout: elements of equal
        (nx, ny, nth) are pushed forward together."""
        if getattr(self, "_coords", None) is None:
            X = np.empty(self.N)
            Y = np.empty(self.N)
            T = np.empty(self.N)
            cols = self.elem_col
            shape = np.stack([self.col_ndofs[cols, 0], self.col_ndofs[cols, 1], self.cell_ndof], axis=1)
            for nx, ny, nt in np.unique(shape, axis=0):
                es = np.nonzero((shape[:, 0] == nx) & (shape[:, 1] == ny) & (shape[:, 2] == nt))[0]
                ci = cols[es]
                xx = push(self.col_pos[ci, 0][:, None], self.col_pos[ci, 2][:, None], quad(0, int(nx))[0][None, :])
                yy = push(self.col_pos[ci, 1][:, None], self.col_pos[ci, 3][:, None], quad(0, int(ny))[0][None, :])
                th = push(self.cell_pos[es, 0][:, None], self.cell_pos[es, 1][:, None], quad(1, int(nt))[0][None, :])
                n = int(nx * ny * nt)
                idx = self.elem_off[es][:, None] + np.arange(n)[None, :]
                full = (len(es), int(nx), int(ny), int(nt))
                X[idx] = np.broadcast_to(xx[:, :, None, None], full).reshape(len(es), n)
                Y[idx] = np.broadcast_to(yy[:, None, :, None], full).reshape(len(es), n)
                T[idx] = np.broadcast_to(th[:, None, None, :], full).reshape(len(es), n)
            for a in (X, Y, T):
                a.setflags(write=False)
            self._coords = (X, Y, T)
        return self._coords

    def signatures(self):
        """Distinct column angular meshes: col_sig[ci] and, per signature, the
        concatenated angular nodes of its cells."""
        sig_of = {}
        col_sig = np.zeros(self.ncols, dtype=np.int32)
        sig_nodes = []
        for ci in range(self.ncols):
            e0, e1 = int(self.col_elem_start[ci]), int(self.col_elem_start[ci + 1])
            key = tuple((float(self.cell_pos[e, 0]), float(self.cell_pos[e, 1]), int(self.cell_ndof[e]))
                        for e in range(e0, e1))
            s = sig_of.get(key)
            if s is None:
                s = len(sig_nodes)
                sig_of[key] = s
                sig_nodes.append(np.concatenate([self.cell_nodes(e) for e in range(e0, e1)]))
            col_sig[ci] = s
        return col_sig, sig_nodes


class SampledCoeffs:
    """kappa, sigma at the column nodes and Phi per column angular mesh."""

    def __init__(self, layout, kappa, sigma, Phi):
        self.kappa = np.ascontiguousarray(layout.sample_spatial(kappa), dtype=np.float64)
        self.sigma = np.ascontiguousarray(layout.sample_spatial(sigma), dtype=np.float64)
        self.col_sig, nodes = layout.signatures()
        blocks = []
        for th in nodes:
            blocks.append(np.ascontiguousarray(
                np.broadcast_to(_eval(Phi, th[:, None], th[None, :]), (len(th), len(th))), dtype=np.float64).ravel())
        self.sig_off = np.zeros(len(blocks) + 1, dtype=np.int64)
        np.cumsum([len(b) for b in blocks], out=self.sig_off[1:])
        self.phi = np.concatenate(blocks) if blocks else np.zeros(1)

    def coeffs(self):
        c = _lib.Coeffs()
        c.kappa = _lib.ptr(self.kappa, C.c_double)
        c.sigma = _lib.ptr(self.sigma, C.c_double)
        c.nsig = len(self.sig_off) - 1
        c.sig_off = _lib.ptr(self.sig_off, C.c_int64)
        c.phi = _lib.ptr(self.phi, C.c_double)
        c.col_sig = _lib.ptr(self.col_sig, C.c_int32)
        return c

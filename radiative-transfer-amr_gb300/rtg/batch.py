"""Many independent RT problems solved together on one GPU.

``BatchContext([(mesh, problem), ...])`` concatenates the instances' flattened
meshes into one librtg handle (column and element indices offset, each
instance with its own sampled kappa, sigma and Phi blocks), so every apply and
sweep covers all instances in one launch; ``solve`` runs rtg_solve_batched,
whose Krylov state is per instance.  The reference solves such a set as a
loop of rt.Problem.solve calls (rt/solve.py:21-181)."""

import ctypes as C

import numpy as np

from . import _lib
from .layout import MeshLayout, SampledCoeffs, _eval
from .problem import _stream_ptr, _torch


class BatchContext:
    def __init__(self, instances, device=None):
        torch = _torch()
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.lib = _lib.load()
        self.layouts = [MeshLayout(m) for m, _ in instances]
        self.specs = [p for _, p in instances]
        lays = self.layouts
        col_off = np.cumsum([0] + [L.ncols for L in lays])
        elem_off = np.cumsum([0] + [L.nelem for L in lays])
        self.inst_off = np.cumsum([0] + [L.N for L in lays]).astype(np.int64)
        self.N = int(self.inst_off[-1])
        nbr = []
        for b, L in enumerate(lays):
            a = L.col_nbr.copy()
            a[a >= 0] += col_off[b]
            nbr.append(a)
        self.col_pos = np.ascontiguousarray(np.concatenate([L.col_pos for L in lays]))
        self.col_ndofs = np.ascontiguousarray(np.concatenate([L.col_ndofs for L in lays]))
        self.col_lv = np.ascontiguousarray(np.concatenate([L.col_lv for L in lays]))
        self.col_nbr = np.ascontiguousarray(np.concatenate(nbr))
        self.col_elem_start = np.ascontiguousarray(np.concatenate(
            [L.col_elem_start[:-1] + elem_off[b] for b, L in enumerate(lays)] + [[elem_off[-1]]]).astype(np.int32))
        self.cell_pos = np.ascontiguousarray(np.concatenate([L.cell_pos for L in lays]))
        self.cell_ndof = np.ascontiguousarray(np.concatenate([L.cell_ndof for L in lays]))
        self.cell_lv = np.ascontiguousarray(np.concatenate([L.cell_lv for L in lays]))
        self.cell_idx = np.ascontiguousarray(np.concatenate([L.cell_idx for L in lays]))
        self.cell_quadrant = np.ascontiguousarray(np.concatenate([L.cell_quadrant for L in lays]))
        samp = [SampledCoeffs(L, p.kappa, p.sigma, p.Phi) for L, p in zip(lays, self.specs)]
        self.kappa = np.ascontiguousarray(np.concatenate([s.kappa for s in samp]))
        self.sigma = np.ascontiguousarray(np.concatenate([s.sigma for s in samp]))
        sig_base = np.cumsum([0] + [len(s.sig_off) - 1 for s in samp])
        phi_base = np.cumsum([0] + [int(s.sig_off[-1]) for s in samp])
        self.col_sig = np.ascontiguousarray(np.concatenate(
            [s.col_sig + sig_base[b] for b, s in enumerate(samp)]).astype(np.int32))
        self.sig_off = np.ascontiguousarray(np.concatenate(
            [s.sig_off[:-1] + phi_base[b] for b, s in enumerate(samp)] + [[phi_base[-1]]]).astype(np.int64))
        self.phi = np.ascontiguousarray(np.concatenate([s.phi[:int(s.sig_off[-1])] for s in samp]))
        d = _lib.MeshDesc()
        d.ncols = int(col_off[-1])
        d.nelem = int(elem_off[-1])
        d.col_pos = _lib.ptr(self.col_pos, C.c_double)
        d.col_ndofs = _lib.ptr(self.col_ndofs, C.c_int32)
        d.col_lv = _lib.ptr(self.col_lv, C.c_int32)
        d.col_nbr = _lib.ptr(self.col_nbr, C.c_int32)
        d.col_elem_start = _lib.ptr(self.col_elem_start, C.c_int32)
        d.cell_pos = _lib.ptr(self.cell_pos, C.c_double)
        d.cell_ndof = _lib.ptr(self.cell_ndof, C.c_int32)
        d.cell_lv = _lib.ptr(self.cell_lv, C.c_int32)
        d.cell_idx = _lib.ptr(self.cell_idx, C.c_int32)
        d.cell_quadrant = _lib.ptr(self.cell_quadrant, C.c_int32)
        c = _lib.Coeffs()
        c.kappa = _lib.ptr(self.kappa, C.c_double)
        c.sigma = _lib.ptr(self.sigma, C.c_double)
        c.nsig = len(self.sig_off) - 1
        c.sig_off = _lib.ptr(self.sig_off, C.c_int64)
        c.phi = _lib.ptr(self.phi, C.c_double)
        c.col_sig = _lib.ptr(self.col_sig, C.c_int32)
        h = C.c_void_p()
        _lib.check(self.lib.rtg_create(C.byref(d), C.byref(c), self.device.index, C.byref(h)))
        self.h = h
        info = _lib.Info()
        _lib.check(self.lib.rtg_get_info(self.h, C.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in _lib.Info._fields_}
        assert int(info.ndof) == self.N

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.rtg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def node_values(self, which):
        """Concatenated f (which = "f") or inflow data (which = "g") at the nodes."""
        out = []
        for L, p in zip(self.layouts, self.specs):
            X, Y, T = L.node_coords()
            fn = p.f if which == "f" else p.bcs_dirac[0]
            out.append(np.asarray(np.broadcast_to(_eval(fn, X, Y, T), (L.N,)), dtype=np.float64))
        return np.ascontiguousarray(np.concatenate(out))

    def forcing(self):
        torch = self.torch
        fv = torch.as_tensor(self.node_values("f")).to(self.device)
        out = torch.empty_like(fv)
        _lib.check(self.lib.rtg_weight_forcing(self.h, C.c_void_p(fv.data_ptr()), C.c_void_p(out.data_ptr()),
                                               _stream_ptr()))
        return out

    def inflow(self):
        return self.torch.as_tensor(self.node_values("g")).to(self.device)

    def solve(self, f_dev, g_dev, rtol=1e-10, atol=0., restart=30, max_it=3000, inner_rtol=1e-5,
              max_outer=20, stream=None):
        """All instances at once; returns (u, [info per instance])."""
        torch = self.torch
        nb = len(self.layouts)
        u = torch.zeros(self.N, dtype=torch.float64, device=self.device)
        o = _lib.SolveOpts(method=1, restart=restart, max_it=max_it, rtol=rtol, atol=atol, precond=1,
                           nonzero_guess=0, inner_rtol=inner_rtol, max_outer=max_outer, verbose=0)
        infos = (_lib.SolveInfo * nb)()
        off = np.ascontiguousarray(self.inst_off)
        _lib.check(self.lib.rtg_solve_batched(self.h, nb, _lib.ptr(off, C.c_int64), C.c_void_p(f_dev.data_ptr()),
                                              C.c_void_p(g_dev.data_ptr()), C.c_void_p(u.data_ptr()),
                                              C.byref(o), infos, _stream_ptr(stream)))
        return u, [{k: getattr(infos[b], k) for k, _ in _lib.SolveInfo._fields_} for b in range(nb)]

    def split(self, v):
        """Per-instance views of a concatenated vector."""
        return [v[int(self.inst_off[b]):int(self.inst_off[b + 1])] for b in range(len(self.layouts))]

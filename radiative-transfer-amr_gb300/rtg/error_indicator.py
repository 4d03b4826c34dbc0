"""Error indicators and hp steering of the AMR loop on the GPU.

Mirrors the reference's ``Error_Indicator`` (src/amr/Error_Indicator/
class_Error_Indicator.py:12-28): ``ErrorIndicator(proj, ref_kind, ref_form,
ref_tol)`` with ``error_angular_jump()`` (error/error_angular_jump.py:14-137),
``error_spatial_jump()`` (error/error_spatial_jump.py:17-289),
``col_hp_steer(col_key)`` (col_hp_steer.py:14-64) and
``cell_hp_steer(col_key, cell_key)`` (cell_hp_steer.py:15-48).  After an
``error_*`` call: ``cols[col_key]`` is an ``ErrorIndicatorColumn`` (``error``,
``cells``, ``ref_form``, ``do_ref``) whose ``cells[cell_key]`` are
``ErrorIndicatorCell`` objects, and ``col_max_error``, ``cell_max_error``,
``error`` and ``error_to_resolve`` are set, as in the reference.  The jumps and
the hp estimates run in librtg's kernels (rtg_error_angular_jump,
rtg_error_spatial_jump, rtg_hp_steer); the flags are set on the host in the
reference's loop order.
"""
import ctypes as C
import math

import numpy as np

from . import _lib

INF = float(np.finfo(np.float64).max)   # the reference's consts.INF


class ErrorIndicatorCell:
    def __init__(self, error, ref_form="", do_ref=False):
        self.error = error
        self.ref_form = ref_form
        self.do_ref = do_ref


class ErrorIndicatorColumn:
    def __init__(self, error, cells, ref_form="", do_ref=False):
        self.error = error
        self.cells = cells
        self.ref_form = ref_form
        self.do_ref = do_ref


def _unit_coefficients():
    return (lambda x, y: 1. + 0. * x, lambda x, y: 0. * x, lambda th, ph: 0. * th + 1. / (2. * math.pi))


class ErrorIndicator:
    """``proj``: an ``rtg.Projection`` (or any object with ``mesh`` and
    ``to_vector()``).  ``ctx``: a DeviceContext on the same mesh to reuse
    (for example the one the solve ran on); one with unit coefficients is
    made otherwise (the indicators use only the mesh)."""

    def __init__(self, proj, ref_kind="all", ref_form="hp", ref_tol=(INF, INF), ctx=None):
        from .problem import DeviceContext
        self.proj = proj
        self.ref_kind = ref_kind
        self.ref_form = ref_form
        [self.ang_ref_tol, self.spt_ref_tol] = ref_tol
        self._own = ctx is None
        self.ctx = ctx if ctx is not None else DeviceContext(proj.mesh, *_unit_coefficients())
        self._u = None
        self._lp = None
        self.cols = {}
        self.col_max_error = -INF
        self.cell_max_error = -INF
        self.error = 0.
        self.error_to_resolve = 0.

    # ------------------------------------------------------------- device
    def _u_dev(self):
        if self._u is None:
            self._u = self.ctx.to_device(np.asarray(self.proj.to_vector(), dtype=np.float64))
        return self._u

    def _keys(self):
        lay = self.ctx.layout
        return lay.col_keys, lay.elem_keys

    def _hp(self):
        if self._lp is None:
            torch = self.ctx.torch
            lay = self.ctx.layout
            col_lp = torch.empty(lay.ncols, dtype=torch.float64, device=self.ctx.device)
            cell_lp = torch.empty(lay.nelem, dtype=torch.float64, device=self.ctx.device)
            _lib.check(self.ctx.lib.rtg_hp_steer(self.ctx.h, C.c_void_p(self._u_dev().data_ptr()),
                                                 C.c_void_p(col_lp.data_ptr()), C.c_void_p(cell_lp.data_ptr()),
                                                 None))
            col_keys, elem_keys = self._keys()
            cl, el = col_lp.cpu().numpy(), cell_lp.cpu().numpy()
            self._lp = ({ck: float(cl[i]) for i, ck in enumerate(col_keys)},
                        {ek: float(el[e]) for e, ek in enumerate(elem_keys)})
        return self._lp

    # ---------------------------------------------------------- hp steering
    def col_hp_steer(self, col_key):
        """'p' when lp - 1/2 >= (nx + ny)/2, else 'h' (col_hp_steer.py:56-64)."""
        lp = self._hp()[0][col_key]
        nx, ny = self.proj.mesh.cols[col_key].ndofs[:2]
        return "p" if lp - 0.5 >= 0.5 * (nx + ny) else "h"

    def cell_hp_steer(self, col_key, cell_key):
        """'p' when lp - 1/2 >= nth, else 'h' (cell_hp_steer.py:40-48)."""
        lp = self._hp()[1][(col_key, cell_key)]
        nth = self.proj.mesh.cols[col_key].cells[cell_key].ndofs[0]
        return "p" if lp - 0.5 >= float(nth) else "h"

    # ----------------------------------------------------------- indicators
    def error_angular_jump(self):
        torch = self.ctx.torch
        lay = self.ctx.layout
        ce = torch.empty(lay.nelem, dtype=torch.float64, device=self.ctx.device)
        _lib.check(self.ctx.lib.rtg_error_angular_jump(self.ctx.h, C.c_void_p(self._u_dev().data_ptr()),
                                                       C.c_void_p(ce.data_ptr()), None, None))
        ce = ce.cpu().numpy()
        col_keys, elem_keys = self._keys()
        cols, col_max, cell_max, mesh_err = {}, -INF, -INF, 0.
        e = 0
        for ck in col_keys:
            cells, s = {}, 0.
            while e < len(elem_keys) and elem_keys[e][0] == ck:
                s += ce[e]
                mesh_err += ce[e]
                cells[elem_keys[e][1]] = ErrorIndicatorCell(math.sqrt(ce[e]))
                cell_max = max(cell_max, math.sqrt(ce[e]))
                e += 1
            cols[ck] = ErrorIndicatorColumn(math.sqrt(s), cells)
            col_max = max(col_max, math.sqrt(s))
        self._finish(cols, col_max, cell_max, mesh_err)

    def error_spatial_jump(self):
        torch = self.ctx.torch
        lay = self.ctx.layout
        cc = torch.empty(lay.ncols, dtype=torch.float64, device=self.ctx.device)
        _lib.check(self.ctx.lib.rtg_error_spatial_jump(self.ctx.h, C.c_void_p(self._u_dev().data_ptr()),
                                                       C.c_void_p(cc.data_ptr()), None))
        cc = cc.cpu().numpy()
        col_keys, elem_keys = self._keys()
        cols, col_max, mesh_err = {}, -INF, 0.
        for i, ck in enumerate(col_keys):
            cells = {kk: ErrorIndicatorCell(-INF) for kk in sorted(self.proj.mesh.cols[ck].cells.keys())}
            mesh_err += cc[i]
            cols[ck] = ErrorIndicatorColumn(math.sqrt(cc[i]), cells)
            col_max = max(col_max, math.sqrt(cc[i]))
        self._finish(cols, col_max, -INF, mesh_err)

    def _finish(self, cols, col_max, cell_max, mesh_err):
        """Maxima, mesh error and the refinement flags in the reference's
        loop order (error_angular_jump.py:84-137)."""
        self.cols = cols
        self.col_max_error = col_max
        self.cell_max_error = cell_max
        self.error = math.sqrt(mesh_err)
        self.error_to_resolve = 0.
        ang_thr = self.ang_ref_tol * self.cell_max_error
        spt_thr = self.spt_ref_tol * self.col_max_error
        for ck in sorted(cols.keys()):
            col = cols[ck]
            if self.ref_kind in ("spt", "all"):
                if col.error >= spt_thr:
                    col.do_ref = True
                    self.error_to_resolve += col.error
                    col.ref_form = self.col_hp_steer(ck) if self.ref_form == "hp" else self.ref_form
                else:
                    col.do_ref = False
            if self.ref_kind in ("ang", "all"):
                for kk in sorted(col.cells.keys()):
                    cell = col.cells[kk]
                    if cell.error >= ang_thr:
                        cell.do_ref = True
                        self.error_to_resolve += cell.error
                        cell.ref_form = self.cell_hp_steer(ck, kk) if self.ref_form == "hp" else self.ref_form
                    else:
                        cell.do_ref = False

    def close(self):
        if self._own and self.ctx is not None:
            self.ctx.close()
        self.ctx = None

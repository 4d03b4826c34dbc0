"""CPU oracle for the AMR error indicators -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy, the reference's indicator methods of
src/amr/Error_Indicator (jasonltorchinsky/radiative-transfer-amr):
``error_angular_jump`` (error/error_angular_jump.py:14-137),
``error_spatial_jump`` (error/error_spatial_jump.py:17-289), ``col_hp_steer``
(col_hp_steer.py:14-64) and ``cell_hp_steer`` (cell_hp_steer.py:15-48), with the
refinement flags they set.  It is the checker for librtg's indicator kernels:
only ``tests/`` and the CPU-baseline leg of ``bench.py`` may use it.  It is
pinned against fixtures the reference itself produced
(tests/golden/make_golden_amr.py).

Inputs: a mesh with the reference's attributes and a vector u in the global
DOF order (sorted column keys, sorted cell keys, beta = nth*ny*i + nth*j + a).
"""

import math

import numpy as np
from scipy.special import eval_legendre

from . import rt_oracle as O

INF = float(np.finfo(np.float64).max)   # consts/__init__.py: INF = np.finfo(REAL).max


def cell_vals(mesh, u, L=None):
    """{(col_key, cell_key): u as an [nx, ny, nth] array} (Projection.from_vector)."""
    L = L or O.Layout(mesh)
    out = {}
    for (ck, kk) in L.elems:
        col = mesh.cols[ck]
        nx, ny = col.ndofs[0], col.ndofs[1]
        nth = col.cells[kk].ndofs[0]
        o = L.off[(ck, kk)]
        out[(ck, kk)] = np.asarray(u[o:o + nx * ny * nth], dtype=np.float64).reshape(nx, ny, nth)
    return out


def angular_jump(mesh, u):
    """Squared errors: per cell 1/4 sum wx wy 0.5 (jump_low^2 + jump_up^2) at
    the cell's theta ends against the neighbour cells ``nhbr_keys`` [low, up];
    per column the sum over its cells (error_angular_jump.py:27-82)."""
    V = cell_vals(mesh, u)
    tops, bots = {}, {}
    for (ck, kk), v in V.items():
        nth = v.shape[2]
        tb, _ = O.lg_nodes(nth)
        top = np.zeros(v.shape[:2])
        bot = np.zeros(v.shape[:2])
        for a in range(nth):
            top += v[:, :, a] * O.lag(tb, a, 1.)
            bot += v[:, :, a] * O.lag(tb, a, -1.)
        tops[(ck, kk)] = top
        bots[(ck, kk)] = bot
    cell_err2, col_err2 = {}, {}
    for ck in sorted(mesh.cols.keys()):
        col = mesh.cols[ck]
        nx, ny = col.ndofs[0], col.ndofs[1]
        _, wx = O.lgl_nodes(nx)
        _, wy = O.lgl_nodes(ny)
        W = wx.reshape(nx, 1) * wy.reshape(1, ny)
        s = 0.
        for kk in sorted(col.cells.keys()):
            lo, up = col.cells[kk].nhbr_keys[0], col.cells[kk].nhbr_keys[1]
            jl = (bots[(ck, kk)] - tops[(ck, lo)]) ** 2
            ju = (tops[(ck, kk)] - bots[(ck, up)]) ** 2
            e = 0.25 * np.sum(W * 0.5 * (jl + ju))
            cell_err2[(ck, kk)] = e
            s += e
        col_err2[ck] = s
    return cell_err2, col_err2


def _face_trace(v, F, own):
    """The face-F trace of an [nx, ny, nth] cell array; own=False gives the
    facing trace of the neighbour (error_spatial_jump.py:140-185)."""
    if not own:
        F = (F + 2) % 4
    return {0: v[-1, :, :], 1: v[:, -1, :], 2: v[0, :, :], 3: v[:, 0, :]}[F]


def spatial_jump(mesh, u):
    """Squared column errors: the trace jumps against every facing neighbour
    cell projected on the finer face interval's LGL rule (max node count) x
    the smaller angular cell's LG rule, summed and divided by perimeter * 2 pi
    (error_spatial_jump.py:33-233)."""
    V = cell_vals(mesh, u)
    out = {}
    for ck0 in sorted(mesh.cols.keys()):
        c0 = mesh.cols[ck0]
        x00, y00, x10, y10 = c0.pos
        perim = 2. * (x10 - x00) + 2. * (y10 - y00)
        jump = 0.
        for F in range(4):
            for ck1 in [k for k in dict.fromkeys(c0.nhbr_keys[F]) if k is not None]:
                c1 = mesh.cols[ck1]
                x01, y01, x11, y11 = c1.pos
                if F % 2 == 0:
                    a0, b0, a1, b1 = y00, y10, y01, y11
                    n0, n1 = c0.ndofs[1], c1.ndofs[1]
                else:
                    a0, b0, a1, b1 = x00, x10, x01, x11
                    n0, n1 = c0.ndofs[0], c1.ndofs[0]
                aA, bA, dA = (a0, b0, b0 - a0) if (b0 - a0) <= (b1 - a1) else (a1, b1, b1 - a1)
                nB = max(n0, n1)
                sB, wB = O.lgl_nodes(nB)
                xf = O.push(aA, bA, sB)
                psi0 = O.lag_mat(O.lgl_nodes(n0)[0], O.pull(a0, b0, xf))   # [n0, nB]
                psi1 = O.lag_mat(O.lgl_nodes(n1)[0], O.pull(a1, b1, xf))
                for kk0 in sorted(c0.cells.keys()):
                    cell0 = c0.cells[kk0]
                    t00, t10 = cell0.pos
                    u0 = _face_trace(V[(ck0, kk0)], F, True)
                    for kk1 in O.nbr_cells(mesh, ck0, kk0, ck1):
                        if kk1 is None:
                            continue
                        cell1 = c1.cells[kk1]
                        t01, t11 = cell1.pos
                        u1 = _face_trace(V[(ck1, kk1)], F, False)
                        gA, gB, dG = (t00, t10, t10 - t00) if (t10 - t00) <= (t11 - t01) else (t01, t11, t11 - t01)
                        nH = max(cell0.ndofs[0], cell1.ndofs[0])
                        sH, wH = O.lg_nodes(nH)
                        th = O.push(gA, gB, sH)
                        xsi0 = O.lag_mat(O.lg_nodes(cell0.ndofs[0])[0], O.pull(t00, t10, th))
                        xsi1 = O.lag_mat(O.lg_nodes(cell1.ndofs[0])[0], O.pull(t01, t11, th))
                        p0 = psi0.T @ u0 @ xsi0
                        p1 = psi1.T @ u1 @ xsi1
                        jump += (dA * dG / 4.) * np.sum(wB.reshape(nB, 1) * wH.reshape(1, nH) * (p0 - p1) ** 2)
        out[ck0] = (1. / (perim * 2. * O.PI)) * jump
    return out


def col_lp(mesh, u, ck, V=None):
    """Legendre-decay estimate of the angle-integrated solution of column ck
    (col_hp_steer.py:14-56)."""
    V = V or cell_vals(mesh, u)
    col = mesh.cols[ck]
    nx, ny = col.ndofs[0], col.ndofs[1]
    xb, wx = O.lgl_nodes(nx)
    yb, wy = O.lgl_nodes(ny)
    uh = np.zeros((nx, ny))
    for kk in sorted(col.cells.keys()):
        cell = col.cells[kk]
        _, wt = O.lg_nodes(cell.ndofs[0])
        uh += (cell.pos[1] - cell.pos[0]) / 2. * np.sum(wt * V[(ck, kk)], axis=2)
    W = wx.reshape(nx, 1) * wy.reshape(1, ny) * uh
    Lx = eval_legendre(nx - 1, xb)
    jj = np.arange(ny)
    Ly = np.array([eval_legendre(j, yb) for j in jj])           # [ny(j), ny(q)]
    a_x = (2. * nx - 1.) * (2. * jj + 1.) / 4. * (Lx @ W @ Ly.T)
    ax2 = np.float64(np.sum(a_x ** 2 * (2. / (2. * jj + 1.))))   # numpy scalars: x/0 -> inf as in the reference
    ii = np.arange(nx)
    Lxi = np.array([eval_legendre(i, xb) for i in ii])
    Lyn = eval_legendre(ny - 1, yb)
    a_y = (2. * ii + 1.) * (2. * ny - 1.) / 4. * (Lxi @ W @ Lyn)
    ay2 = np.float64(np.sum(a_y ** 2 * (2. / (2. * ii + 1.))))
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = np.log((2. * nx - 1.) / (2 * ax2)) / (2. * np.log(nx - 1.))
        t1 = np.log((2. * ny - 1.) / (2 * ay2)) / (2. * np.log(ny - 1.))
    return float(0.5 * (t0 + t1))


def cell_lp(mesh, u, ck, kk, V=None):
    """Legendre-decay estimate of the space-integrated solution of one cell
    (cell_hp_steer.py:15-40)."""
    V = V or cell_vals(mesh, u)
    col = mesh.cols[ck]
    nx, ny = col.ndofs[0], col.ndofs[1]
    x0, y0, x1, y1 = col.pos
    _, wx = O.lgl_nodes(nx)
    _, wy = O.lgl_nodes(ny)
    nth = col.cells[kk].ndofs[0]
    tb, wt = O.lg_nodes(nth)
    uh = (x1 - x0) * (y1 - y0) / 4. * np.sum(wx.reshape(nx, 1, 1) * wy.reshape(1, ny, 1) * V[(ck, kk)], axis=(0, 1))
    a = (2. * nth - 1.) / 2. * np.float64(np.sum(wt * uh * eval_legendre(nth - 1, tb)))
    asq = a * a * (2. / (2. * nth - 1.))
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.log((2. * nth - 1.) / (2 * asq)) / (2. * np.log(nth - 1.)))


def col_form(mesh, ck, lp):
    col = mesh.cols[ck]
    return "p" if lp - 0.5 >= 0.5 * (col.ndofs[0] + col.ndofs[1]) else "h"   # col_hp_steer.py:58-64


def cell_form(mesh, ck, kk, lp):
    return "p" if lp - 0.5 >= float(mesh.cols[ck].cells[kk].ndofs[0]) else "h"   # cell_hp_steer.py:42-48


def indicator(mesh, u, kind, ref_kind="all", ref_form="hp", ref_tol=(INF, INF)):
    """The reference's indicator state after error_angular_jump ("ang") or
    error_spatial_jump ("spt"): {"cols": {ck: {"error", "do_ref", "ref_form",
    "cells": {kk: {"error", "do_ref", "ref_form"}}}}, "col_max_error",
    "cell_max_error", "error", "error_to_resolve"} (error_angular_jump.py:
    84-137, error_spatial_jump.py:235-289)."""
    ang_tol, spt_tol = ref_tol
    V = cell_vals(mesh, u)
    cols = {}
    col_max, cell_max, mesh_err = -INF, -INF, 0.
    if kind == "ang":
        ce2, _ = angular_jump(mesh, u)
        for ck in sorted(mesh.cols.keys()):
            cells, s = {}, 0.
            for kk in sorted(mesh.cols[ck].cells.keys()):
                e2 = ce2[(ck, kk)]
                s += e2
                mesh_err += e2
                cells[kk] = {"error": math.sqrt(e2), "do_ref": False, "ref_form": ""}
                cell_max = max(cell_max, math.sqrt(e2))
            cols[ck] = {"error": math.sqrt(s), "do_ref": False, "ref_form": "", "cells": cells}
            col_max = max(col_max, math.sqrt(s))
    else:
        cc2 = spatial_jump(mesh, u)
        for ck in sorted(mesh.cols.keys()):
            cells = {kk: {"error": -INF, "do_ref": False, "ref_form": ""} for kk in sorted(mesh.cols[ck].cells.keys())}
            mesh_err += cc2[ck]
            cols[ck] = {"error": math.sqrt(cc2[ck]), "do_ref": False, "ref_form": "", "cells": cells}
            col_max = max(col_max, math.sqrt(cc2[ck]))
    res = 0.
    ang_thr, spt_thr = ang_tol * cell_max, spt_tol * col_max
    for ck in sorted(mesh.cols.keys()):
        c = cols[ck]
        if ref_kind in ("spt", "all"):
            if c["error"] >= spt_thr:
                c["do_ref"] = True
                res += c["error"]
                c["ref_form"] = col_form(mesh, ck, col_lp(mesh, u, ck, V)) if ref_form == "hp" else ref_form
            else:
                c["do_ref"] = False
        if ref_kind in ("ang", "all"):
            for kk in sorted(mesh.cols[ck].cells.keys()):
                cc = c["cells"][kk]
                if cc["error"] >= ang_thr:
                    cc["do_ref"] = True
                    res += cc["error"]
                    cc["ref_form"] = cell_form(mesh, ck, kk, cell_lp(mesh, u, ck, kk, V)) if ref_form == "hp" \
                        else ref_form
                else:
                    cc["do_ref"] = False
    return {"cols": cols, "col_max_error": col_max, "cell_max_error": cell_max, "error": math.sqrt(mesh_err),
            "error_to_resolve": res}

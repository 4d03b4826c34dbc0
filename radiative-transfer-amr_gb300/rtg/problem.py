"""Drop-in ``Problem`` for the reference's ``rt.Problem`` (rt/class_Problem.py:11-32).

Same constructor (kappa, sigma, Phi, f, bcs_dirac) and method names.  The
matrix builders return ``DeviceOperator`` objects in place of PETSc ``Mat``:
they apply the reference's matrices matrix-free on the GPU (``mult``), combine
with ``+``/``-`` like the reference's drivers do
(experiments/test-rt/experiment.py:77-287: ``ma - sc + (bc - ic)``), and can be
materialised as scipy matrices for small meshes.  ``solve`` returns
``[Projection, convergence_info, matrix_info]`` with the keys of
rt/solve.py:171-181.  All compute runs in librtg on the GPU; there is no CPU
path.
"""

import ctypes as C
import time

import numpy as np

from . import _lib
from .layout import MeshLayout, SampledCoeffs, _eval
from .projection import Projection

EPS = float(np.finfo(np.float64).resolution)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("rtg needs a CUDA device; none is available")
    return torch


def _stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def mesh_fingerprint(mesh):
    parts = []
    for ck in sorted(mesh.cols.keys()):
        col = mesh.cols[ck]
        parts.append((ck, tuple(col.ndofs), tuple(col.pos),
                      tuple(tuple(x) for x in col.nhbr_keys),
                      tuple((kk, col.cells[kk].ndofs[0], col.cells[kk].quadrant, tuple(col.cells[kk].pos))
                            for kk in sorted(col.cells.keys()))))
    return hash(tuple(parts))


class DeviceContext:
    """One librtg handle: the operator tables of one mesh and coefficient set."""

    def __init__(self, mesh, kappa, sigma, Phi, device=None):
        torch = _torch()
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.lib = _lib.load()
        self.layout = MeshLayout(mesh)
        self.sampled = SampledCoeffs(self.layout, kappa, sigma, Phi)
        desc, keep = self.layout.mesh_desc()
        co = self.sampled.coeffs()
        h = C.c_void_p()
        _lib.check(self.lib.rtg_create(C.byref(desc), C.byref(co), self.device.index, C.byref(h)))
        self.h = h
        info = _lib.Info()
        _lib.check(self.lib.rtg_get_info(self.h, C.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in _lib.Info._fields_}
        self.N = int(info.ndof)
        self._mask = None

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.rtg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- vectors
    def to_device(self, v, dtype=None):
        torch = self.torch
        dtype = dtype or torch.float64
        if isinstance(v, torch.Tensor):
            t = v.to(device=self.device, dtype=dtype)
        else:
            t = torch.as_tensor(np.array(v, dtype=np.float64), dtype=dtype).to(self.device)
        t = t.contiguous()
        if t.numel() != self.N:
            raise ValueError("vector length {} != ndof {}".format(t.numel(), self.N))
        return t

    def apply(self, flags, x, y=None, prec=_lib.RTG_FP64, stream=None):
        torch = self.torch
        dt = torch.float64 if prec == _lib.RTG_FP64 else torch.float32
        x = self.to_device(x, dt)
        if y is None:
            y = torch.empty(self.N, dtype=dt, device=self.device)
        _lib.check(self.lib.rtg_apply(self.h, flags, prec, C.c_void_p(x.data_ptr()),
                                      C.c_void_p(y.data_ptr()), _stream_ptr(stream)))
        return y

    def precondition(self, r, z=None, prec=_lib.RTG_FP64, stream=None):
        """z = P^{-1} r with the upwind transport sweep."""
        torch = self.torch
        dt = torch.float64 if prec == _lib.RTG_FP64 else torch.float32
        r = self.to_device(r, dt)
        if z is None:
            z = torch.empty(self.N, dtype=dt, device=self.device)
        _lib.check(self.lib.rtg_precondition(self.h, prec, C.c_void_p(r.data_ptr()),
                                             C.c_void_p(z.data_ptr()), _stream_ptr(stream)))
        return z

    def interior_mask(self):
        if self._mask is None:
            torch = self.torch
            m = torch.empty(self.N, dtype=torch.uint8, device=self.device)
            _lib.check(self.lib.rtg_interior_mask(self.h, C.c_void_p(m.data_ptr()), _stream_ptr()))
            self._mask = m.bool()
        return self._mask

    def node_values(self, fn):
        X, Y, T = self.layout.node_coords()
        return np.ascontiguousarray(_eval(fn, X, Y, T), dtype=np.float64)

    def forcing(self, f):
        """Weighted forcing vector on the device (rt/forcing_vector.py:103-155)."""
        torch = self.torch
        fv = self.to_device(self.node_values(f))
        out = torch.empty_like(fv)
        _lib.check(self.lib.rtg_weight_forcing(self.h, C.c_void_p(fv.data_ptr()),
                                               C.c_void_p(out.data_ptr()), _stream_ptr()))
        return out

    def inflow(self, bcs_dirac):
        """Inflow data at every node (rt/boundary_conditions_vector.py:101-207)."""
        bcs, dirac = bcs_dirac
        # any(dirac), as the reference tests it: truthiness, so a lone Dirac
        # coordinate of 0.0 keeps the sampled branch
        # (rt/boundary_conditions_vector.py:142)
        if not any(dirac):
            return self.to_device(self.node_values(bcs))
        return self.to_device(_dirac_inflow(self.layout, bcs, dirac))

    def solve(self, f_dev, g_dev, method=0, restart=50, max_it=5000, rtol=1e-12, atol=0.,
              precond=0, x0=None, inner_rtol=1e-6, max_outer=20, stream=None, hist_cap=8192):
        torch = self.torch
        u = torch.zeros(self.N, dtype=torch.float64, device=self.device) if x0 is None else \
            self.to_device(x0).clone()
        o = _lib.SolveOpts(method=method, restart=restart, max_it=max_it, rtol=rtol, atol=atol,
                           precond=precond, nonzero_guess=0 if x0 is None else 1,
                           inner_rtol=inner_rtol, max_outer=max_outer, verbose=0)
        info = _lib.SolveInfo()
        hist = np.zeros(hist_cap)
        _lib.check(self.lib.rtg_solve(self.h, C.c_void_p(f_dev.data_ptr()), C.c_void_p(g_dev.data_ptr()),
                                      C.c_void_p(u.data_ptr()), C.byref(o), C.byref(info),
                                      _lib.ptr(hist, C.c_double), hist_cap, _stream_ptr(stream)))
        out = {k: getattr(info, k) for k, _ in _lib.SolveInfo._fields_}
        out["history"] = hist[:info.hist_len].copy()
        return u, out

    def extreme_singular_values(self, stream=None):
        """[emax, emin] of the last solve's last Arnoldi cycle: the singular
        values of its Givens-reduced Hessenberg factor, the estimate the
        reference reads with ksp.computeExtremeSingularValues()
        (rt/solve.py:110-115).  [1, 1] when no cycle ran, as PETSc returns."""
        n = C.c_int32()
        _lib.check(self.lib.rtg_solve_hessenberg(self.h, None, 0, C.byref(n), _stream_ptr(stream)))
        if n.value == 0:
            return [1.0, 1.0]
        R = np.zeros(n.value * n.value)
        _lib.check(self.lib.rtg_solve_hessenberg(self.h, _lib.ptr(R, C.c_double), R.size, C.byref(n),
                                                 _stream_ptr(stream)))
        sv = np.linalg.svd(R.reshape(n.value, n.value).T, compute_uv=False)
        return [float(sv[0]), float(sv[-1])]


def _dirac_inflow(lay, bcs, dirac):
    """Point-source inflow data (rt/boundary_conditions_vector.py:142-196),
    including its bookkeeping: a cell wholly outside the Dirac point in every
    given coordinate writes nothing and does not advance the write position."""
    from .layout import quad
    out = np.zeros(lay.N)
    for ci in range(lay.ncols):
        x0, y0, x1, y1 = lay.col_pos[ci]
        e0, e1 = int(lay.col_elem_start[ci]), int(lay.col_elem_start[ci + 1])
        pos = int(lay.elem_off[e0])
        xx, yy = lay.col_nodes(ci)
        nx, ny = len(xx), len(yy)
        for e in range(e0, e1):
            th0, th1 = lay.cell_pos[e]
            nth = int(lay.cell_ndof[e])
            lims = [(x0, x1, quad(0, nx)[0], xx), (y0, y1, quad(0, ny)[0], yy),
                    (th0, th1, quad(1, nth)[0], lay.cell_nodes(e))]
            inside = [True, True, True]
            fac, crd = [], []
            for d in range(3):
                a, b, tnod, phys = lims[d]
                n = len(tnod)
                if dirac[d] is not None and not (dirac[d] < a or b < dirac[d]):
                    sb = -1.0 + 2.0 / (b - a) * (dirac[d] - a)
                    lv = []
                    for m in range(n):
                        if -1.0 - 1.e-14 <= sb <= 1.0 + 1.e-14:
                            r = 1.
                            for j in range(n):
                                if j != m:
                                    r *= (sb - tnod[j]) / (tnod[m] - tnod[j])
                        else:
                            r = 0.
                        lv.append(max(0.0, r))
                    fac.append(np.array(lv))
                    crd.append(np.full(n, float(dirac[d])))
                else:
                    if dirac[d] is not None:
                        inside[d] = False
                    fac.append(np.ones(n))
                    crd.append(phys)
            if any(inside):
                bv = np.broadcast_to(_eval(bcs, crd[0][:, None, None], crd[1][None, :, None],
                                           crd[2][None, None, :]), (nx, ny, nth))
                v = bv * fac[0][:, None, None] * fac[1][None, :, None] * fac[2][None, None, :]
                out[pos:pos + nx * ny * nth] = v.reshape(-1)
                pos += nx * ny * nth
    return out


class DeviceOperator:
    """Linear combination of the reference's RT matrices, applied on the GPU."""

    def __init__(self, ctx, terms):
        self.ctx = ctx
        self.terms = list(terms)   # [(coef, flags)]

    def getSize(self):
        return (self.ctx.N, self.ctx.N)

    @property
    def shape(self):
        return (self.ctx.N, self.ctx.N)

    def _combine(self, other, sign):
        if not isinstance(other, DeviceOperator) or other.ctx is not self.ctx:
            return NotImplemented
        return DeviceOperator(self.ctx, self.terms + [(sign * c, f) for c, f in other.terms])

    def __add__(self, other):
        return self._combine(other, 1.)

    def __sub__(self, other):
        return self._combine(other, -1.)

    def __neg__(self):
        return DeviceOperator(self.ctx, [(-c, f) for c, f in self.terms])

    def __mul__(self, a):
        return DeviceOperator(self.ctx, [(a * c, f) for c, f in self.terms])

    __rmul__ = __mul__

    def _normalised(self):
        acc = {}
        for c, f in self.terms:
            acc[f] = acc.get(f, 0.) + c
        return {f: c for f, c in acc.items() if c != 0.}

    def mult(self, x, y=None, prec=_lib.RTG_FP64):
        """y = Op x.  numpy in -> numpy out; torch (device) in -> torch out."""
        torch = self.ctx.torch
        as_numpy = not isinstance(x, torch.Tensor)
        terms = self._normalised()
        system = {_lib.RTG_BC: 1., _lib.RTG_IC: -1., _lib.RTG_MASS | _lib.RTG_SCAT: 1.}
        if terms == system:
            terms = {_lib.RTG_SYSTEM: 1.}
        out = None
        for f, c in terms.items():
            t = self.ctx.apply(f, x, prec=prec)
            out = t.mul_(c) if out is None else out.add_(t, alpha=c)
        if out is None:
            out = torch.zeros(self.ctx.N, dtype=torch.float64, device=self.ctx.device)
        if y is not None:
            if isinstance(y, torch.Tensor):
                y.copy_(out)
            else:
                y[:] = out.cpu().numpy()
            return y
        return out.cpu().numpy() if as_numpy else out

    def __matmul__(self, x):
        return self.mult(x)

    def to_scipy(self, block=256):
        """Materialise as a scipy CSR matrix by applying to unit vectors
        (meant for meshes of a few thousand DOF)."""
        import scipy.sparse as sp
        torch = self.ctx.torch
        N = self.ctx.N
        cols = []
        for j0 in range(0, N, block):
            j1 = min(N, j0 + block)
            for j in range(j0, j1):
                e = torch.zeros(N, dtype=torch.float64, device=self.ctx.device)
                e[j] = 1.
                cols.append(self.mult(e))
        D = torch.stack(cols, dim=1).cpu().numpy()
        return sp.csr_matrix(D)


# pc_type names (the reference's PETSc names and this library's own) -> the
# preconditioner rtg_solve applies (Problem.solve documents the mapping)
PC_TYPES = {"none": 0, "sweep": 1, "bjacobi": 1, "kaczmarz": 1, "dsa": 2, "learned": 3}


class Problem:
    """rt.Problem with the GPU behind it (rt/class_Problem.py:11-32)."""

    def __init__(self, kappa, sigma, Phi, f, bcs_dirac):
        self.kappa = kappa
        self.sigma = sigma
        self.Phi = Phi
        self.f = f
        self.bcs_dirac = bcs_dirac
        self._ctx = {}

    def context(self, mesh):
        key = (id(mesh), mesh_fingerprint(mesh))
        ctx = self._ctx.get(key)
        if ctx is None:
            self._ctx.clear()
            ctx = DeviceContext(mesh, self.kappa, self.sigma, self.Phi)
            self._ctx[key] = ctx
        return ctx

    # builders (rt/mass_matrix.py:23 and siblings)
    def mass_matrix(self, mesh, **kwargs):
        return DeviceOperator(self.context(mesh), [(1., _lib.RTG_MASS)])

    def scattering_matrix(self, mesh, **kwargs):
        return DeviceOperator(self.context(mesh), [(1., _lib.RTG_SCAT)])

    def preconditioner_matrix(self, mesh, **kwargs):
        """[M - S, None] as rt/preconditioner_matrix.py:22-114 returns."""
        return [DeviceOperator(self.context(mesh), [(1., _lib.RTG_MASS | _lib.RTG_SCAT)]), None]

    def interior_convection_matrix(self, mesh, **kwargs):
        return DeviceOperator(self.context(mesh), [(1., _lib.RTG_IC)])

    def boundary_convection_matrix(self, mesh, **kwargs):
        return DeviceOperator(self.context(mesh), [(1., _lib.RTG_BC)])

    def forcing_vector(self, mesh, **kwargs):
        t = self.context(mesh).forcing(self.f)
        return t if kwargs.get("as_tensor") else t.cpu().numpy()

    def boundary_conditions_vector(self, mesh, **kwargs):
        t = self.context(mesh).inflow(self.bcs_dirac)
        return t if kwargs.get("as_tensor") else t.cpu().numpy()

    def solve(self, mesh, **kwargs):
        """Solve the split system (rt/solve.py:21-181).

        kwargs: ksp_type "gmres" or "fgmres" (FP64 GMRES, the plain method;
        with a fixed preconditioner right-preconditioned GMRES and FGMRES build
        the same iterates) or "mixed" (FP32 GMRES inside FP64 iterative
        refinement); pc_type (below); restart (50), max_it (5000), rtol (1e-12;
        the reference asks PETSc for 1e-15), atol (0), x0 ("forcing" = start
        from f_I as the reference does, or "zero").

        pc_type: the reference hands its string to PETSc (rt/solve.py:93-95);
        here every name maps to a GPU preconditioner.  "bjacobi" (PETSc's
        default, block Jacobi over ranks) and "kaczmarz" (row projections in
        row order, the two-scatterer inputs' choice,
        experiments/two-strong-scatterers/input.json:4-7) both map to the
        upwind transport sweep: for the upwind DG operator the sweep is the
        block Gauss-Seidel pass in flow order, the transport form of a
        row-action sweep, and the algebraic methods themselves (a dense
        row-by-row pass) have no GPU form worth shipping.  "none", "sweep",
        "dsa" (with the column diffusion correction) and "learned" (with the
        learned correction) name the others."""
        opts = {"verbose": False, "ksp_type": "gmres", "pc_type": "sweep", "restart": 50,
                "max_it": 5000, "rtol": 1e-12, "atol": 0., "x0": "forcing",
                "inner_rtol": 1e-6}
        opts.update(kwargs)
        t0 = time.perf_counter()
        ctx = self.context(mesh)
        f_dev = ctx.forcing(self.f)
        g_dev = ctx.inflow(self.bcs_dirac)
        method = {"gmres": 0, "mixed": 1, "fgmres": 0}.get(opts["ksp_type"])
        if method is None:
            raise ValueError("unsupported ksp_type {}".format(opts["ksp_type"]))
        # PETSc's "bjacobi" default maps to the sweep, the GPU preconditioner;
        # "dsa" adds the column diffusion correction, "learned" the learned
        # correction (a network set with rtg.learned.set_params)
        precond = PC_TYPES.get(opts["pc_type"])
        if precond is None:
            raise ValueError("unsupported pc_type {}".format(opts["pc_type"]))
        x0 = f_dev if opts["x0"] == "forcing" else None
        u, info = ctx.solve(f_dev, g_dev, method=method, restart=int(opts["restart"]),
                            max_it=int(opts["max_it"]), rtol=float(opts["rtol"]),
                            atol=float(opts["atol"]), x0=x0, inner_rtol=float(opts["inner_rtol"]),
                            precond=precond)
        uh = Projection(mesh)
        uh.from_vector(u.cpu().numpy())
        hist = info["history"]
        converged_reason = 2 if info["converged"] else -3      # PETSc RTOL / DIVERGED_ITS
        convergence_info = {"converged_reason": converged_reason,
                            "convergence_history": hist.tolist(),
                            "iteration_number": int(info["iterations"]),
                            "res_f": float(info["res_f"]),
                            "res_best": float(np.min(hist)) if len(hist) else float(info["res_f"]),
                            "rtol": float(opts["rtol"]), "atol": float(opts["atol"]),
                            "divtol": float(np.sqrt(np.finfo(np.float64).max)),
                            "max_it": int(opts["max_it"])}
        matrix_info = {"ndof": ctx.N, "ndof_interior": int(ctx.info["ndof_interior"]),
                       "ncoupling": int(ctx.info["ncoupling"]),
                       "extreme_singular_values": ctx.extreme_singular_values(),
                       "solve_seconds": time.perf_counter() - t0,
                       "fp64_applies": int(info["fp64_applies"]),
                       "fp32_applies": int(info["fp32_applies"])}
        if opts["verbose"]:
            print("rtg solve: N={} iterations={} res_f={:.3e} converged={}".format(
                ctx.N, info["iterations"], info["res_f"], bool(info["converged"])))
        return [uh, convergence_info, matrix_info]

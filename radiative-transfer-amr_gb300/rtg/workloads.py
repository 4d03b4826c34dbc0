"""Seeded synthetic RT problems and hp meshes.

Each problem is the five callables the reference's ``rt.Problem`` takes
(rt/class_Problem.py:12-23): kappa(x, y) (total extinction), sigma(x, y)
(scattering), Phi(th, phi), f(x, y, th), and ``bcs_dirac = [bcs, dirac]``.
Coefficient callables accept numpy arrays (broadcasting) and scalars.

The mesh recipes only call ``Mesh(...)``, ``ref_mesh``, ``ref_col`` and
``ref_cell``, so the same recipe applied to the reference's ``dg.mesh.Mesh``
produces the same mesh.

The Henyey-Greenstein phase function is the one the reference's experiment
drivers supply (experiments/two-strong-scatterers/problem.py:36-43):
Phi(th, phi) = (1 - g^2) / N_g / (1 + g^2 - 2 g cos(th - phi))^(3/2), with N_g
its integral over [0, 2 pi] computed by adaptive quadrature to 1e-9.
"""

import math
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from .mesh import Mesh

PI = math.pi


@dataclass
class RTProblemSpec:
    name: str
    kappa: Callable
    sigma: Callable
    Phi: Callable
    f: Callable
    bcs_dirac: list
    u_exact: Optional[Callable] = None
    meta: dict = field(default_factory=dict)


def _quad(fn, a, b):
    from scipy.integrate import quad
    val, _ = quad(fn, a, b, epsabs=1.e-9, epsrel=1.e-9, limit=100, maxp1=100)
    return val


def hg_phase(g):
    """Reference-normalised HG kernel with exponent 3/2 (see module docstring)."""
    g = float(g)
    norm = _quad(lambda d: (1. - g ** 2) / (1 + g ** 2 - 2. * g * np.cos(d)) ** (3. / 2.),
                 0., 2. * PI)

    def Phi(th, phi):
        return ((1. - g ** 2) / norm) / (1 + g ** 2 - 2. * g * np.cos(th - phi)) ** (3. / 2.)

    Phi.g = g
    Phi.norm = norm
    return Phi


# ----------------------------------------------------------------- problems
def manufactured_problem(Lx=1., Ly=1., sigma_t=1.1, sigma_s=0.5, g=0.8, width=0.05):
    """u = exp(-((x-Lx/2)^2 + (y-Ly/2)^2)/width) (1 + cos(th)/2), constant
    coefficients; f = s.grad u + sigma_t u - sigma_s int Phi u dth', inflow data u.

    int_0^{2pi} Phi(th, th') (1 + cos th'/2) dth' = 1 + (c1/2) cos th with
    c1 = int Phi(0, d) cos d dd, because Phi integrates to one and depends on
    th - th' only."""
    Phi = hg_phase(g)
    c1 = _quad(lambda d: Phi(0., d) * np.cos(d), 0., 2. * PI)
    xc, yc = Lx / 2., Ly / 2.

    def X(x, y):
        return np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / width)

    def u(x, y, th):
        return X(x, y) * (1. + 0.5 * np.cos(th))

    def kappa(x, y):
        return sigma_t + 0. * (x + y)

    def sigma(x, y):
        return sigma_s + 0. * (x + y)

    def f(x, y, th):
        Xv = X(x, y)
        dX = -2. * Xv / width
        Th = 1. + 0.5 * np.cos(th)
        prop = (np.cos(th) * (x - xc) + np.sin(th) * (y - yc)) * dX * Th
        return prop + sigma_t * Xv * Th - sigma_s * Xv * (1. + 0.5 * c1 * np.cos(th))

    def bcs(x, y, th):
        return u(x, y, th)

    return RTProblemSpec("manufactured", kappa, sigma, Phi, f, [bcs, [None, None, None]],
                         u_exact=u, meta={"g": g, "c1": c1})


def smooth_variable_problem(Lx=1., Ly=1., g=0.6):
    """Variable kappa/sigma, smooth forcing and inflow data (no exact solution);
    exercises every operator term with non-constant coefficients."""
    Phi = hg_phase(g)

    def kappa(x, y):
        return 1.5 + 0.5 * np.sin(PI * x / Lx) * np.cos(PI * y / Ly)

    def sigma(x, y):
        return 0.6 * kappa(x, y)

    def f(x, y, th):
        return (1. + x * y) * (1. + 0.3 * np.sin(th) + 0.2 * np.cos(2. * th))

    def bcs(x, y, th):
        return np.exp(-x) * (1. + 0.5 * np.cos(th - 0.3)) + 0.1 * y

    return RTProblemSpec("smooth_variable", kappa, sigma, Phi, f, [bcs, [None, None, None]],
                         meta={"g": g})


def point_inflow_problem(Lx=3., Ly=2., g=0.6, dirac=(0.0, None, 0.3)):
    """The smooth variable coefficients with a point-source inflow: ``dirac``
    gives the Dirac position in x, y and/or th (None where the data are
    sampled), the reference's ``bcs_dirac = [bcs, dirac]`` form
    (rt/boundary_conditions_vector.py:142-196).  The default puts the source
    at x = 0 in th = 0.3; a coordinate of 0.0 is a real position inside the
    branch even though the reference's any(dirac) test alone would skip it."""
    base = smooth_variable_problem(Lx, Ly, g)
    return RTProblemSpec("point_inflow", base.kappa, base.sigma, base.Phi, base.f,
                         [base.bcs_dirac[0], list(dirac)], meta={"g": g, "dirac": list(dirac)})


def gaussian_bump_problem(Lx=3., Ly=2., amp=0.9, width=0.15, xc=1.5, yc=1.0, g=0.9):
    """Single adaptive problem: sigma_s = amp exp(-r^2 / (2 width^2)) centred at
    (xc, yc), sigma_t = sigma_s + 0.01, isotropic inflow 1 on x = 0 for
    th in (-pi/4, pi/4), zero elsewhere, no interior source."""
    Phi = hg_phase(g)

    def sigma(x, y):
        return amp * np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / (2. * width ** 2))

    def kappa(x, y):
        return sigma(x, y) + 0.01

    def f(x, y, th):
        return 0. * (x + y + th)

    def bcs(x, y, th):
        x = np.asarray(x, dtype=float)
        th = np.asarray(th, dtype=float)
        beam = (th < PI / 4.) | (th > 7. * PI / 4.)
        return np.where((x == 0.) & beam, 1., 0.)

    return RTProblemSpec("gaussian_bump", kappa, sigma, Phi, f, [bcs, [None, None, None]],
                         meta={"g": g})


def two_disc_problem(Lx=2., Ly=2., g=0.95, discs=((0.6, 0.6), (1.4, 1.4)), rad=0.2, sigma_s=50.):
    """Two strong scatterers: discs of radius 0.2 at (0.6, 0.6) and (1.4, 1.4)
    with sigma_s = 50, sigma_t = 50.1 inside; background sigma_t = 0.1,
    sigma_s = 0.01; beam inflow on y = 0 for |x - 1| < 0.25, |th - pi/2| < pi/8.
    (discs, rad and sigma_s vary it for the learned correction's training
    family; sigma_t = sigma_s + 0.1 inside.)"""
    Phi = hg_phase(g)
    discs = tuple(tuple(d) for d in discs)
    sig_in, kap_in = float(sigma_s), float(sigma_s) + 0.1

    def inside(x, y):
        x = np.asarray(x, dtype=float)
        y = np.asarray(y, dtype=float)
        m = np.zeros(np.broadcast(x, y).shape, dtype=bool)
        for (cx, cy) in discs:
            m |= ((x - cx) ** 2 + (y - cy) ** 2) <= rad ** 2
        return m

    def kappa(x, y):
        return np.where(inside(x, y), kap_in, 0.1)

    def sigma(x, y):
        return np.where(inside(x, y), sig_in, 0.01)

    def f(x, y, th):
        return 0. * (x + y + th)

    def bcs(x, y, th):
        x = np.asarray(x, dtype=float)
        y = np.asarray(y, dtype=float)
        th = np.asarray(th, dtype=float)
        on = (y == 0.) & (np.abs(x - 1.) < 0.25) & (np.abs(th - PI / 2.) < PI / 8.)
        return np.where(on, 1., 0.)

    return RTProblemSpec("two_disc", kappa, sigma, Phi, f, [bcs, [None, None, None]],
                         meta={"g": g, "discs": discs, "radius": rad})


def gaussian_source_problem(sigma_t, ratio, g, Lx=1., Ly=1., xs=0.5, ys=0.5, ws=0.1):
    """Batched instance: constant sigma_t, sigma_s = ratio * sigma_t, Gaussian
    isotropic source at (xs, ys), vacuum inflow."""
    Phi = hg_phase(g)

    def kappa(x, y):
        return sigma_t + 0. * (x + y)

    def sigma(x, y):
        return ratio * sigma_t + 0. * (x + y)

    def f(x, y, th):
        return np.exp(-((x - xs) ** 2 + (y - ys) ** 2) / ws ** 2) + 0. * th

    def bcs(x, y, th):
        return 0. * (x + y + th)

    return RTProblemSpec("gaussian_source", kappa, sigma, Phi, f, [bcs, [None, None, None]],
                         meta={"g": g, "sigma_t": sigma_t, "ratio": ratio})


# -------------------------------------------------------------- mesh recipes
def uniform_mesh(Ls, n, nref_ang, nref_spt, mesh_cls=Mesh, pbcs=(False, False)):
    """``Mesh(Ls, pbcs, [n, n, n])`` refined uniformly ``nref_ang`` times in angle
    then ``nref_spt`` times in space (experiments/manufactured-solution/mesh.py:18-28)."""
    mesh = mesh_cls(list(Ls), list(pbcs), [n, n, n], True)
    for _ in range(nref_ang):
        mesh.ref_mesh(kind="ang", form="h")
    for _ in range(nref_spt):
        mesh.ref_mesh(kind="spt", form="h")
    return mesh


def config1_mesh(mesh_cls=Mesh):
    """[0,1]^2, 4x4 columns x 4 angular cells, 4 nodes per dimension (4096 DOF)."""
    return uniform_mesh([1., 1.], 4, 2, 2, mesh_cls)


def hanging_hp_mesh(mesh_cls=Mesh):
    """The scripted refinement sequence of the reference's mesh test
    (tests/test_dg/test_mesh/test_Mesh.py:40-66): non-conforming spatial and
    angular neighbours with mixed degrees."""
    mesh = mesh_cls([1., 2.], [False, False], [2, 3, 4], True)
    for ck, kind, form in zip([0, 0, 0, 1, 10, 48], ["ang", "ang", "spt", "spt", "spt", "spt"],
                              ["h", "h", "h", "h", "hp", "hp"]):
        mesh.ref_col(col_key=ck, kind=kind, form=form)
    for kk, form in zip([3, 7, 15], ["h", "hp", "hp"]):
        mesh.ref_cell(col_key=204, cell_key=kk, form=form)
    return mesh


def quadrant_free_mesh(mesh_cls=Mesh):
    """Two angular cells per column ([0, pi], [pi, 2 pi]): cells outside any
    single quadrant, so no face is treated as outflow for them."""
    mesh = mesh_cls([1., 1.], [False, False], [3, 3, 2], True)
    mesh.ref_mesh(kind="ang", form="h")
    mesh.ref_mesh(kind="spt", form="h")
    mesh.ref_mesh(kind="spt", form="h")
    mesh.ref_col(col_key=sorted(mesh.cols.keys())[5], kind="spt", form="p")
    return mesh


def periodic_mesh(mesh_cls=Mesh):
    """Periodic in x, vacuum-bounded in y."""
    mesh = mesh_cls([1., 1.], [True, False], [3, 3, 3], True)
    mesh.ref_mesh(kind="ang", form="h")
    mesh.ref_mesh(kind="ang", form="h")
    mesh.ref_mesh(kind="spt", form="h")
    return mesh


def random_hp_mesh(Ls, n0, nth0, rounds, seed, frac_spt=0.3, frac_ang=0.2,
                   p_prob=0.4, n_max=7, nref_ang=2, nref_spt=2, mesh_cls=Mesh,
                   ndof_cap=None):
    """Seeded random hp refinement: start from a uniform mesh, then for each
    round pick leaf columns to refine in space (h or p) and leaf cells to refine
    in angle (h or p), with ``numpy.random.default_rng(seed)``.  Refinement
    goes through the mesh's own ``ref_col``/``ref_cell`` (2:1 balance kept).
    Degrees are capped at ``n_max`` nodes; ``ndof_cap`` stops early."""
    rng = np.random.default_rng(seed)
    mesh = mesh_cls(list(Ls), [False, False], [n0, n0, nth0], True)
    for _ in range(nref_ang):
        mesh.ref_mesh(kind="ang", form="h")
    for _ in range(nref_spt):
        mesh.ref_mesh(kind="spt", form="h")
    for _ in range(rounds):
        keys = sorted(mesh.cols.keys())
        pick = rng.random(len(keys)) < frac_spt
        forms = rng.random(len(keys)) < p_prob
        for ck, pk, pf in zip(keys, pick, forms):
            if not pk or ck not in mesh.cols:
                continue
            col = mesh.cols[ck]
            if pf and col.ndofs[0] < n_max:
                mesh.ref_col(ck, kind="spt", form="p")
            elif not pf:
                mesh.ref_col(ck, kind="spt", form="h")
        keys = sorted(mesh.cols.keys())
        for ck in keys:
            if ck not in mesh.cols:
                continue
            ckeys = sorted(mesh.cols[ck].cells.keys())
            pick = rng.random(len(ckeys)) < frac_ang
            forms = rng.random(len(ckeys)) < p_prob
            for kk, pk, pf in zip(ckeys, pick, forms):
                if not pk or ck not in mesh.cols or kk not in mesh.cols[ck].cells:
                    continue
                cell = mesh.cols[ck].cells[kk]
                if pf and cell.ndofs[0] < n_max:
                    mesh.ref_cell(ck, kk, form="p")
                elif not pf and cell.lv < 6:
                    mesh.ref_cell(ck, kk, form="h")
        if ndof_cap is not None and mesh.get_ndof() >= ndof_cap:
            break
    return mesh


def small_random_mesh(mesh_cls=Mesh, seed=3):
    """A few thousand DOF of random hp refinement on [0,3]x[0,2]."""
    return random_hp_mesh([3., 2.], 2, 3, rounds=3, seed=seed, frac_spt=0.35,
                          frac_ang=0.3, n_max=5, nref_ang=2, nref_spt=1,
                          mesh_cls=mesh_cls)


def disc_edge_mesh(mesh_cls=Mesh, seed=0, rounds=3, n0=4, nth0=4, n_max=9, nref_ang=3,
                   nref_spt=3, p_prob=0.35, ang_prob=0.35, max_ang_lv=5, discs=((0.6, 0.6), (1.4, 1.4)),
                   radius=0.2, Ls=(2., 2.), ndof_cap=None):
    """Two-strong-scatterer mesh: uniform start, then seeded refinement of the
    columns that straddle a disc edge (h with probability 1 - p_prob, else p
    up to ``n_max`` nodes) and of the angular cells of those columns (h up to
    level ``max_ang_lv`` or p), all through ref_col/ref_cell (2:1 balance)."""
    rng = np.random.default_rng(seed)
    mesh = mesh_cls(list(Ls), [False, False], [n0, n0, nth0], True)
    for _ in range(nref_ang):
        mesh.ref_mesh(kind="ang", form="h")
    for _ in range(nref_spt):
        mesh.ref_mesh(kind="spt", form="h")

    def near_edge(col):
        x0, y0, x1, y1 = col.pos
        cx, cy = (x0 + x1) / 2., (y0 + y1) / 2.
        half = 0.5 * max(x1 - x0, y1 - y0) * 1.5
        return any(abs(np.hypot(cx - dx, cy - dy) - radius) < half for dx, dy in discs)

    for _ in range(rounds):
        for ck in sorted(mesh.cols.keys()):
            if ck not in mesh.cols or not near_edge(mesh.cols[ck]):
                continue
            col = mesh.cols[ck]
            if rng.random() < p_prob:
                if col.ndofs[0] < n_max:
                    mesh.ref_col(ck, kind="spt", form="p")
            else:
                mesh.ref_col(ck, kind="spt", form="h")
        for ck in sorted(mesh.cols.keys()):
            if ck not in mesh.cols or not near_edge(mesh.cols[ck]):
                continue
            for kk in sorted(mesh.cols[ck].cells.keys()):
                if ck not in mesh.cols or kk not in mesh.cols[ck].cells or rng.random() >= ang_prob:
                    continue
                cell = mesh.cols[ck].cells[kk]
                if rng.random() < 0.5 and cell.ndofs[0] < n_max:
                    mesh.ref_cell(ck, kk, form="p")
                elif cell.lv < max_ang_lv:
                    mesh.ref_cell(ck, kk, form="h")
        if ndof_cap is not None and mesh.get_ndof() >= ndof_cap:
            break
    return mesh


def config5_mesh(mesh_cls=Mesh, seed=0, scale=1.0):
    """Large two-strong-scatterer mesh on [0,2]^2: 16x16 columns of 5x5 nodes
    and 32 angular cells of 5 nodes to start, then four rounds of seeded
    refinement concentrated at the disc edges (h or p in space up to 9 nodes
    per dimension, h up to 64 cells or p up to 9 nodes in angle), about 8e6 DOF
    at scale 1 (``scale`` < 1 gives the same recipe with fewer rounds).

    The angular start is set by the phase function, not by cost: with HG
    g = 0.95 the discrete kernel (dth/2 w) Phi of a coarse angular mesh is far
    from conservative (largest eigenvalue of D^1/2 Phi D^1/2, D = diag(dth/2 w):
    2.18 on 8 cells of 5 nodes, 1.20 on 16, 1.01 on 32), so inside the discs
    (sigma_s / sigma_t = 0.998) a coarse mesh makes kappa - sigma lambda
    strongly negative: a multiplying medium whose linear system GMRES cannot
    solve in any reasonable number of iterations.  On 32 cells the system is
    within 0.4 of that limit and sweep-preconditioned GMRES converges in about
    40-50 iterations."""
    rounds = 4 if scale >= 1.0 else max(0, int(round(4 * scale)))
    return disc_edge_mesh(mesh_cls=mesh_cls, seed=seed, rounds=rounds, n0=5, nth0=5, n_max=9,
                          nref_ang=5, nref_spt=4, ang_prob=0.1, max_ang_lv=6)


def config5_small_mesh(mesh_cls=Mesh, seed=0, rounds=1):
    """The two-strong-scatterer recipe at a size the CPU oracle assembles in
    seconds: 8x8 columns of 2x2 nodes, the same 32 angular cells of 5 nodes,
    ``rounds`` rounds of disc-edge refinement up to 4 nodes per dimension
    (about 6.7e4 DOF at one round)."""
    return disc_edge_mesh(mesh_cls=mesh_cls, seed=seed, rounds=rounds, n0=2, nth0=5, n_max=4,
                          nref_ang=5, nref_spt=3, ang_prob=0.1, max_ang_lv=6)


def batch_instance(seed, mesh_cls=Mesh, max_cols=64, max_cells=16, n_range=(2, 8)):
    """One instance of the batched workload, drawn from ``seed``: [0,1]^2,
    8..64 spatial columns (random leaf h-refinement of a 2x2 start), 4..16
    angular cells per column (at least 4 so that every cell lies in one
    quadrant), a single degree p in [1, 7] (2..8 nodes) for x, y and th,
    sigma_t ~ U(0.5, 5), sigma_s / sigma_t ~ U(0.1, 0.99), HG g ~ U(0, 0.95),
    Gaussian isotropic source, vacuum inflow."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(n_range[0], n_range[1] + 1))
    target_cols = int(rng.integers(8, max_cols + 1))
    target_cells = int(rng.integers(4, max_cells + 1))
    mesh = mesh_cls([1., 1.], [False, False], [n, n, n], True)
    mesh.ref_mesh(kind="ang", form="h")
    mesh.ref_mesh(kind="ang", form="h")
    mesh.ref_mesh(kind="spt", form="h")
    while len(mesh.cols) + 3 <= target_cols:
        keys = sorted(mesh.cols.keys())
        before = len(mesh.cols)
        mesh.ref_col(keys[int(rng.integers(len(keys)))], kind="spt", form="h")
        if len(mesh.cols) > max_cols:
            break
        if len(mesh.cols) == before:
            break
    # refine the same angular cell in every column until the target count
    for _ in range(64):
        c0 = mesh.cols[sorted(mesh.cols.keys())[0]]
        if len(c0.cells) >= target_cells:
            break
        cand = [k for k in sorted(c0.cells.keys()) if c0.cells[k].lv < 4]
        if not cand:
            break
        kk = cand[int(rng.integers(len(cand)))]
        for ck in sorted(mesh.cols.keys()):
            if kk in mesh.cols[ck].cells:
                mesh.ref_cell(ck, kk, form="h")
    sigma_t = float(rng.uniform(0.5, 5.))
    ratio = float(rng.uniform(0.1, 0.99))
    g = float(rng.uniform(0., 0.95))
    xs, ys = (float(v) for v in rng.uniform(0.3, 0.7, size=2))
    return mesh, gaussian_source_problem(sigma_t, ratio, g, xs=xs, ys=ys)


def disc_family_instance(seed, mesh_cls=Mesh):
    """One problem of the learned correction's two-scatterer family: one or
    two discs (centres U([0.4, 1.6]^2), radius U(0.1, 0.3)), sigma_s
    log-uniform in [2, 50] inside (sigma_t = sigma_s + 0.1), HG g in
    U(0.7, 0.95), the two-scatterer beam inflow, on the resolved-angle
    disc-edge recipe at one refinement round (8x8 columns of 2x2 or 3x3 nodes,
    32 angular cells of 5 nodes; about 7e4 to 1.5e5 DOF)."""
    rng = np.random.default_rng(104729 + seed)
    nd = int(rng.integers(1, 3))
    discs = tuple((float(a), float(b)) for a, b in rng.uniform(0.4, 1.6, size=(nd, 2)))
    rad = float(rng.uniform(0.1, 0.3))
    sig = float(np.exp(rng.uniform(np.log(2.), np.log(50.))))
    g = float(rng.uniform(0.7, 0.95))
    n0 = int(rng.integers(2, 4))
    mesh = disc_edge_mesh(mesh_cls=mesh_cls, seed=seed, rounds=1, n0=n0, nth0=5, n_max=n0 + 2, nref_ang=5,
                          nref_spt=3, ang_prob=0.1, max_ang_lv=6, discs=discs, radius=rad)
    spec = two_disc_problem(g=g, discs=discs, rad=rad, sigma_s=sig)
    spec.meta.update({"seed": seed, "sigma_s": sig})
    return mesh, spec


def config2_mesh(mesh_cls=Mesh, seed=0):
    """Single adaptive problem mesh: [0,3]x[0,2], six rounds of seeded random
    hp refinement, nodes per dimension in [3, 7] (degree 2..6), about 2e5 DOF."""
    return random_hp_mesh([3., 2.], 3, 3, rounds=6, seed=seed, frac_spt=0.3,
                          frac_ang=0.12, p_prob=0.5, n_max=7, nref_ang=2,
                          nref_spt=2, mesh_cls=mesh_cls)


def config4_instance(seed, mesh_cls=Mesh, rounds=3, n_max=6):
    """One problem of the learned-preconditioner family (config-2 type): the
    Gaussian-bump scatterer on [0,3]x[0,2] with seeded amplitude
    (log-uniform in [0.5, 50]), width (U(0.1, 0.3)), centre
    (U([0.6, 2.4] x [0.5, 1.5])) and HG g (U(0, 0.95)), sigma_t = sigma_s +
    0.01, the config-2 beam inflow, on a seeded random hp mesh of the config-2
    recipe with fewer rounds (about 2e4 to 1e5 DOF at rounds=3)."""
    rng = np.random.default_rng(7919 + seed)
    amp = float(np.exp(rng.uniform(np.log(0.5), np.log(50.))))
    width = float(rng.uniform(0.1, 0.3))
    xc = float(rng.uniform(0.6, 2.4))
    yc = float(rng.uniform(0.5, 1.5))
    g = float(rng.uniform(0., 0.95))
    mesh = random_hp_mesh([3., 2.], 3, 3, rounds=rounds, seed=seed, frac_spt=0.3, frac_ang=0.12,
                          p_prob=0.5, n_max=n_max, nref_ang=2, nref_spt=2, mesh_cls=mesh_cls)
    spec = gaussian_bump_problem(amp=amp, width=width, xc=xc, yc=yc, g=g)
    spec.meta.update({"amp": amp, "width": width, "xc": xc, "yc": yc, "seed": seed})
    return mesh, spec

"""GPU operator parity: every reference matrix applied matrix-free by librtg
matches the reference-assembled scipy matrix (golden fixtures) on random
vectors.  FP64 tolerance: 1e-12 relative (2-norm of the product)."""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


@pytest.fixture(scope="module", params=golden_io.CASES)
def case(request):
    from rtg import Problem
    name = request.param
    g = golden_io.load(name)
    mesh_fn, prob_fn = golden_io.problem(name)
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    return name, g, mesh, prob


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _vectors(n, k=3, seed=0):
    rng = np.random.default_rng(seed)
    vs = [rng.standard_normal(n) for _ in range(k)]
    vs.append(np.ones(n))
    return vs


def test_components(case):
    name, g, mesh, prob = case
    ops = {"M": prob.mass_matrix(mesh), "S": prob.scattering_matrix(mesh),
           "MS": prob.preconditioner_matrix(mesh)[0], "IC": prob.interior_convection_matrix(mesh),
           "BC": prob.boundary_convection_matrix(mesh)}
    for nm, op in ops.items():
        for v in _vectors(len(g["f"])):
            err = _rel(op.mult(v), g[nm] @ v)
            assert err < TOL64, (name, nm, err)


def test_system_operator(case):
    name, g, mesh, prob = case
    ma_sc, _ = prob.preconditioner_matrix(mesh)
    A = (prob.boundary_convection_matrix(mesh) - prob.interior_convection_matrix(mesh)) + ma_sc
    for v in _vectors(len(g["f"]), seed=1):
        err = _rel(A.mult(v), g["A"] @ v)
        assert err < TOL64, (name, err)


def test_masked_system_and_fp32(case):
    from rtg import _lib
    name, g, mesh, prob = case
    ctx = prob.context(mesh)
    mask = g["mask"]
    for v in _vectors(len(g["f"]), seed=2):
        vi = np.where(mask, v, 0.)
        ref = np.where(mask, g["A"] @ vi, 0.)
        y = ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, vi).cpu().numpy()
        assert _rel(y, ref) < TOL64
        y32 = ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, vi, prec=_lib.RTG_FP32).cpu().numpy()
        assert _rel(y32, ref) < TOL32, _rel(y32, ref)
    np.testing.assert_array_equal(ctx.interior_mask().cpu().numpy(), mask)
    assert int(ctx.info["ndof_interior"]) == int(mask.sum())


def test_vectors(case):
    name, g, mesh, prob = case
    f = prob.forcing_vector(mesh)
    b = prob.boundary_conditions_vector(mesh)
    assert _rel(f, g["f"]) < 1e-13
    assert _rel(b, g["g"]) < 1e-13 or np.linalg.norm(g["g"]) == 0.


def test_split_merge_roundtrip(case):
    import ctypes as C
    import torch
    from rtg import _lib
    name, g, mesh, prob = case
    ctx = prob.context(mesh)
    x = ctx.to_device(np.arange(len(g["f"]), dtype=np.float64))
    ni = int(ctx.info["ndof_interior"])
    xi = torch.empty(ni, dtype=torch.float64, device=ctx.device)
    _lib.check(ctx.lib.rtg_split_vector(ctx.h, C.c_void_p(x.data_ptr()), C.c_void_p(xi.data_ptr()), None))
    gg = ctx.to_device(-np.ones(len(g["f"])))
    out = torch.empty_like(x)
    _lib.check(ctx.lib.rtg_merge_vectors(ctx.h, C.c_void_p(xi.data_ptr()), C.c_void_p(gg.data_ptr()),
                                         C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    ref = np.where(g["mask"], np.arange(len(g["f"]), dtype=np.float64), -1.)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    np.testing.assert_array_equal(xi.cpu().numpy(), np.nonzero(g["mask"])[0].astype(np.float64))


def test_to_scipy_small():
    from rtg import Problem
    g = golden_io.load("periodic")
    mesh_fn, prob_fn = golden_io.problem("periodic")
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    B = prob.boundary_convection_matrix(mesh).to_scipy()
    D = (B - g["BC"]).toarray()
    assert np.abs(D).max() <= 1e-14 * abs(g["BC"]).max()


def test_sweep_preconditioner_properties(case):
    """P^{-1} r: finite, zero at inflow-boundary DOFs, repeatable across calls
    (the sentinel fill before every sweep), FP32 (BF16 block inverses) within
    1e-2 of FP64, linear."""
    import torch
    from rtg import _lib
    name, g, mesh, prob = case
    ctx = prob.context(mesh)
    rng = np.random.default_rng(5)
    r = np.where(g["mask"], rng.standard_normal(len(g["f"])), 0.)
    z1 = ctx.precondition(r).cpu().numpy()
    z2 = ctx.precondition(r).cpu().numpy()
    assert np.all(np.isfinite(z1))
    np.testing.assert_array_equal(z1, z2)
    assert np.all(z1[~g["mask"]] == 0.)
    if name != "quad_none":
        # quad_none's element blocks have no outflow terms and are nearly
        # singular, so FP32 and FP64 sweeps legitimately differ there
        z32 = ctx.precondition(r, prec=_lib.RTG_FP32).cpu().numpy()
        assert np.linalg.norm(z32 - z1) <= 1e-2 * np.linalg.norm(z1)
    z3 = ctx.precondition(2.5 * r).cpu().numpy()
    assert np.linalg.norm(z3 - 2.5 * z1) <= 1e-12 * np.linalg.norm(z3)


@pytest.mark.parametrize("name", [c for c in golden_io.CASES if c != "quad_none"])
def test_sweep_matches_oracle(name):
    """rtg_precondition against the oracle's restatement of the sweep (same
    level order, element blocks from the reference-assembled matrices).  The
    GPU inverts the element blocks in FP32, so agreement is to ~1e-5."""
    from rtg import Problem
    from oracle import rt_oracle as O
    g = golden_io.load(name)
    mesh_fn, prob_fn = golden_io.problem(name)
    spec = prob_fn()
    mesh = mesh_fn()
    o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    P = O.SweepPreconditioner(o, o["layout"])
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    ctx = prob.context(mesh)
    rng = np.random.default_rng(11)
    r = np.where(g["mask"], rng.standard_normal(len(g["f"])), 0.)
    z_ref = P(r)
    z = ctx.precondition(r).cpu().numpy()
    assert np.linalg.norm(z - z_ref) <= 1e-4 * np.linalg.norm(z_ref), np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref)

"""GPU solve parity: the device Krylov solves reproduce the reference's split
system solution (direct solve of the reference-assembled matrix)."""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


# quad_none: every angular cell spans two quadrants, so the reference
# formulation has no outflow face terms and its split system is indefinite
# (eigenvalues with negative real part, cond ~1.4e4); restarted GMRES(50)
# stalls there for the reference's assembled matrix as well (scipy: relative
# residual 0.78 after 10k iterations).  It is covered by the operator parity
# tests and by test_indefinite_case_reports_nonconvergence below.
SOLVE_CASES = [c for c in golden_io.CASES if c != "quad_none"]


@pytest.fixture(scope="module", params=SOLVE_CASES)
def case(request):
    from rtg import Problem
    name = request.param
    g = golden_io.load(name)
    mesh_fn, prob_fn = golden_io.problem(name)
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    return name, g, mesh, prob, spec


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_unpreconditioned_fp64_gmres(case):
    name, g, mesh, prob, _ = case
    if name == "hp_hanging":
        pytest.skip("unpreconditioned GMRES(50) stagnates on this mesh; covered with the sweep")
    uh, conv, minfo = prob.solve(mesh, ksp_type="gmres", pc_type="none", rtol=1e-13, max_it=20000)
    u = uh.to_vector()
    assert conv["converged_reason"] > 0, conv["res_f"]
    assert _rel(u, g["u"]) < 1e-10, _rel(u, g["u"])


def test_sweep_preconditioner_cuts_iterations(case):
    name, g, mesh, prob, _ = case
    _, c0, _ = prob.solve(mesh, pc_type="none", rtol=1e-10, max_it=3000)
    uh, c1, _ = prob.solve(mesh, pc_type="sweep", rtol=1e-10, max_it=3000)
    assert c1["converged_reason"] > 0
    assert c1["iteration_number"] < c0["iteration_number"], (c1["iteration_number"], c0["iteration_number"])
    assert _rel(uh.to_vector(), g["u"]) < 1e-7


def test_plain_fp64_gmres(case):
    name, g, mesh, prob, _ = case
    uh, conv, minfo = prob.solve(mesh, ksp_type="gmres", rtol=1e-14, max_it=20000)
    u = uh.to_vector()
    assert conv["converged_reason"] > 0, conv["res_f"]
    assert _rel(u, g["u"]) < 1e-11, _rel(u, g["u"])
    for key in ("converged_reason", "convergence_history", "iteration_number", "res_f",
                "res_best", "rtol", "atol", "divtol", "max_it"):
        assert key in conv


def test_mixed_precision_ir(case):
    name, g, mesh, prob, _ = case
    uh, conv, minfo = prob.solve(mesh, ksp_type="mixed", rtol=1e-13, max_it=20000)
    u = uh.to_vector()
    assert conv["converged_reason"] > 0
    assert _rel(u, g["u"]) < 1e-10, _rel(u, g["u"])
    assert minfo["fp32_applies"] > minfo["fp64_applies"]


@pytest.mark.parametrize("ksp", ["gmres", "mixed"])
def test_two_level_diffusion_preconditioner(case, ksp):
    """Sweep + column diffusion correction (flexible GMRES) reaches the same
    solution as the direct solve of the reference-assembled system."""
    name, g, mesh, prob, _ = case
    uh, conv, minfo = prob.solve(mesh, ksp_type=ksp, pc_type="dsa", rtol=1e-13, max_it=20000)
    assert conv["converged_reason"] > 0
    assert _rel(uh.to_vector(), g["u"]) < 1e-10, _rel(uh.to_vector(), g["u"])


def test_two_level_on_thick_scatterer():
    """On an optically thick, nearly isotropic scatterer the diffusion
    correction converges to the sweep-preconditioned solution."""
    import torch
    from rtg import DeviceContext, workloads as W
    mesh, _ = W.config4_instance(1, rounds=2)
    spec = W.gaussian_bump_problem(amp=30.0, width=0.3, g=0.1)
    ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    f = ctx.forcing(spec.f)
    gv = ctx.inflow(spec.bcs_dirac)
    u1, i1 = ctx.solve(f, gv, method=0, precond=1, rtol=1e-12, restart=30, max_it=3000)
    u2, i2 = ctx.solve(f, gv, method=0, precond=2, rtol=1e-12, restart=30, max_it=3000)
    assert i1["converged"] and i2["converged"] and i2["coarse"] > 0
    assert float(torch.linalg.norm(u2 - u1) / torch.linalg.norm(u1)) < 1e-9


def test_manufactured_error_cfg1():
    from rtg import Problem
    g = golden_io.load("cfg1")
    mesh_fn, prob_fn = golden_io.problem("cfg1")
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    uh, conv, _ = prob.solve(mesh, rtol=1e-12)
    from rtg.layout import MeshLayout
    lay = MeshLayout(mesh)
    X, Y, T = lay.node_coords()
    w = prob.mass_matrix(mesh).mult(np.ones(lay.N)) / 1.1
    ue = spec.u_exact(X, Y, T)
    err = np.sqrt(np.sum(w * (uh.to_vector() - ue) ** 2) / np.sum(w * ue ** 2))
    np.testing.assert_allclose(err, float(g["rel_l2_err_exact"]), rtol=1e-8)


def test_indefinite_case_reports_nonconvergence():
    from rtg import Problem
    mesh_fn, prob_fn = golden_io.problem("quad_none")
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    uh, conv, _ = prob.solve(mesh, rtol=1e-12, max_it=500)
    assert conv["converged_reason"] < 0
    assert conv["iteration_number"] <= 500
    assert np.all(np.isfinite(uh.to_vector()))


def test_reference_solver_parameters(case):
    """The two-scatterer inputs' solver choice (ksp_type fgmres, pc_type
    kaczmarz: experiments/two-strong-scatterers/input.json:4-7) goes through,
    and matrix_info carries the extreme singular values (rt/solve.py:110-115)."""
    name, g, mesh, prob, _ = case
    uh, conv, minfo = prob.solve(mesh, ksp_type="fgmres", pc_type="kaczmarz", rtol=1e-13, max_it=20000)
    assert conv["converged_reason"] > 0
    assert _rel(uh.to_vector(), g["u"]) < 1e-10
    emax, emin = minfo["extreme_singular_values"]
    assert np.isfinite(emax) and np.isfinite(emin) and emax >= emin > 0.


def test_extreme_singular_values_match_arnoldi():
    """Unpreconditioned FP64 GMRES stopped after one 20-step cycle: the
    singular values of the cycle's Hessenberg from the library equal those of
    a numpy Arnoldi (classical Gram-Schmidt, one projection per step, as the
    library and PETSc's GMRES orthogonalise) on the reference-assembled A_II
    from r0 = b."""
    from rtg import Problem
    g = golden_io.load("cfg1")
    mesh_fn, prob_fn = golden_io.problem("cfg1")
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    _, conv, minfo = prob.solve(mesh, pc_type="none", restart=30, max_it=20, rtol=1e-30, x0="zero")
    assert conv["iteration_number"] == 20
    mask = g["mask"]
    I, B = np.nonzero(mask)[0], np.nonzero(~mask)[0]
    A = g["A"].tocsr()
    AII = A[I][:, I]
    b = g["f"][I] - A[I][:, B] @ g["g"][B]
    V = [b / np.linalg.norm(b)]
    H = np.zeros((21, 20))
    for j in range(20):
        w = AII @ V[j]
        h = np.array([v @ w for v in V])
        w = w - sum(hq * v for hq, v in zip(h, V))
        H[:j + 1, j] = h
        H[j + 1, j] = np.linalg.norm(w)
        V.append(w / H[j + 1, j])
    sv = np.linalg.svd(H, compute_uv=False)
    emax, emin = minfo["extreme_singular_values"]
    assert abs(emax - sv[0]) < 1e-10 * sv[0], (emax, sv[0])
    assert abs(emin - sv[-1]) < 1e-8 * sv[0], (emin, sv[-1])

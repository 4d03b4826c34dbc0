"""Parity with the CPU oracle at benchmark sizes.

Two problems the oracle assembles in seconds: the single adaptive problem at
its full size (2.2e5 DOF, p up to 6, hanging nodes) and the two-strong-
scatterer recipe at 6.7e4 DOF (32 angular cells of 5 nodes, disc-edge hp
refinement; the recipe of the 8e6-DOF problem with fewer rounds and
columns).  The oracle's solution is its own sweep-preconditioned scipy GMRES
to a relative residual of 1e-13 (on the adaptive problem it agrees with a
direct solve of the same system to 1.4e-14).

* the FP64 system apply (split-system rows) matches A @ x to 1e-12 relative;
* forcing and inflow vectors match to 1e-13;
* the plain FP64 solve matches the oracle's solution to 1e-10 (quadrature-
  weighted relative L2 norm);
* the mixed-precision solve (FP32 inner GMRES, FP64 refinement) reaches the
  1e-8 error target against the oracle's solution;
* the sweep preconditioner matches the oracle's sweep to 1e-4 in FP64 (FP32-
  built element inverses) and to 1e-2 in FP32 (their BF16 copies).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_APPLY = 1e-12
TOL_PLAIN = 1e-10
ERR_TARGET = 1e-8


def _problems():
    from rtg import workloads as W
    return {"adaptive_2e5": (W.config2_mesh, W.gaussian_bump_problem),
            "two_disc_6.7e4": (lambda: W.config5_small_mesh(rounds=1), W.two_disc_problem)}


@pytest.fixture(scope="module", params=["adaptive_2e5", "two_disc_6.7e4"])
def sized(request):
    from oracle import rt_oracle as O
    from rtg import Problem
    mesh_fn, spec_fn = _problems()[request.param]
    mesh, spec = mesh_fn(), spec_fn()
    o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    u_ref, its, info = O.solve_sweep_gmres(o, o["layout"], rtol=1e-13, maxiter=400)
    A_II, _, rhs, I, _ = O.split_system(o["A"], o["f"], o["g"], o["mask"])
    res = np.linalg.norm(rhs - A_II @ u_ref[I]) / np.linalg.norm(rhs)
    assert res < 1e-12, ("oracle solve", res)
    w = O.l2_weights(mesh, o["layout"])
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    ctx = prob.context(mesh)
    yield request.param, o, u_ref, w, ctx, spec
    ctx.close()


def _wrel(u, ref, w):
    return float(np.sqrt(np.sum(w * (u - ref) ** 2) / np.sum(w * ref ** 2)))


def test_fp64_apply_matches_oracle(sized):
    from rtg import _lib
    name, o, _, _, ctx, _ = sized
    mask = o["mask"]
    A = o["A"]
    rng = np.random.default_rng(11)
    for k in range(3):
        v = rng.standard_normal(o["N"])
        vi = np.where(mask, v, 0.)
        ref = np.where(mask, A @ vi, 0.)
        y = ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, vi).cpu().numpy()
        err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
        assert err < TOL_APPLY, (name, k, err)
    y = ctx.apply(_lib.RTG_SYSTEM, v).cpu().numpy()
    assert np.linalg.norm(y - A @ v) / np.linalg.norm(A @ v) < TOL_APPLY


def test_vectors_match_oracle(sized):
    name, o, _, _, ctx, spec = sized
    f = ctx.forcing(spec.f).cpu().numpy()
    g = ctx.inflow(spec.bcs_dirac).cpu().numpy()
    assert np.linalg.norm(f - o["f"]) <= 1e-13 * max(np.linalg.norm(o["f"]), 1e-300)
    assert np.linalg.norm(g - o["g"]) <= 1e-13 * np.linalg.norm(o["g"])


def test_plain_solve_matches_oracle(sized):
    name, o, u_ref, w, ctx, spec = sized
    f, g = ctx.forcing(spec.f), ctx.inflow(spec.bcs_dirac)
    u, info = ctx.solve(f, g, method=0, precond=1, rtol=1e-13, max_it=20000)
    assert info["converged"]
    err = _wrel(u.cpu().numpy(), u_ref, w)
    assert err < TOL_PLAIN, (name, err)


def test_mixed_solve_reaches_target_against_oracle(sized):
    name, o, u_ref, w, ctx, spec = sized
    f, g = ctx.forcing(spec.f), ctx.inflow(spec.bcs_dirac)
    u, info = ctx.solve(f, g, method=1, precond=1, rtol=1e-10, max_it=20000, restart=30, inner_rtol=1e-5)
    assert info["converged"]
    err = _wrel(u.cpu().numpy(), u_ref, w)
    assert err < ERR_TARGET, (name, err, info["iterations"], info["outer"])


def test_sweep_matches_oracle_sized(sized):
    """The sweep preconditioner in both precisions against the oracle's
    restatement (block LU per element and angular node, level order) on a
    random residual: these meshes hold conforming elements whose couplings
    take the sweep's diagonal-mortar path, and hanging and angularly refined
    ones that take the mortar sums.  The GPU inverts the element blocks in
    FP32, so the FP64 sweep agrees to about 1e-5 (bound 1e-4); the FP32 sweep
    reads BF16 copies of them, about 2e-3 (bound 1e-2)."""
    from oracle import rt_oracle as O
    from rtg import _lib
    name, o, _, _, ctx, _ = sized
    P = O.SweepPreconditioner(o, o["layout"])
    rng = np.random.default_rng(23)
    r = np.where(o["mask"], rng.standard_normal(len(o["mask"])), 0.)
    z_ref = P(r)
    for prec, tol in ((_lib.RTG_FP64, 1e-4), (_lib.RTG_FP32, 1e-2)):
        z = ctx.precondition(r, prec=prec).double().cpu().numpy()
        err = np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref)
        assert err <= tol, (name, prec, err)

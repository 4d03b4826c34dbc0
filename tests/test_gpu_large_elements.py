"""Parity on a mesh that forces the large-element code paths: 9 nodes per
dimension and 16 angular cells per column (144 angular nodes), so the apply
reads the column's angular scattering matrix through L2 instead of shared
memory and the sweep's element block inverses (9 x 81 x 81) are too large to
prefetch.  Coefficients: the two-strong-scatterer problem."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    from rtg import Problem, workloads as W
    from oracle import rt_oracle as O
    mesh = W.uniform_mesh([2., 2.], 9, 4, 1)
    spec = W.two_disc_problem()
    o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    return mesh, spec, o, prob


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_large_element_apply(big):
    from rtg import _lib
    mesh, spec, o, prob = big
    ctx = prob.context(mesh)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(o["N"])
    assert _rel(ctx.apply(_lib.RTG_SYSTEM, v).cpu().numpy(), o["A"] @ v) < 1e-12
    v32 = ctx.apply(_lib.RTG_SYSTEM, v, prec=_lib.RTG_FP32).cpu().numpy()
    assert _rel(v32, o["A"] @ v) < 2e-5
    for flag, nm in ((_lib.RTG_SCAT, "S"), (_lib.RTG_IC, "IC"), (_lib.RTG_BC, "BC")):
        assert _rel(ctx.apply(flag, v).cpu().numpy(), o[nm] @ v) < 1e-12, nm


def test_large_element_sweep(big):
    from oracle import rt_oracle as O
    mesh, spec, o, prob = big
    ctx = prob.context(mesh)
    P = O.SweepPreconditioner(o, o["layout"])
    rng = np.random.default_rng(4)
    r = np.where(o["mask"], rng.standard_normal(o["N"]), 0.)
    z_ref = P(r)
    z = ctx.precondition(r).cpu().numpy()
    assert _rel(z, z_ref) < 1e-4


def test_large_element_solve(big):
    """The GPU solution satisfies the reference-assembled split system."""
    from oracle import rt_oracle as O
    mesh, spec, o, prob = big
    uh, conv, _ = prob.solve(mesh, rtol=1e-12, max_it=2000)
    assert conv["converged_reason"] > 0
    A_II, A_IB, rhs, I, B = O.split_system(o["A"], o["f"], o["g"], o["mask"])
    u = uh.to_vector()
    assert np.linalg.norm(A_II @ u[I] - rhs) <= 1e-10 * np.linalg.norm(rhs)
    np.testing.assert_array_equal(u[B], o["g"][B])

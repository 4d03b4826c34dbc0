"""Batched solve: instances concatenated in one handle and solved together
(per-instance Krylov state on the device, one CUDA-graph cycle per restart)
give the same solutions as solving each instance on its own."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_matches_individual_solves():
    from rtg import Problem, workloads as W
    from rtg.batch import BatchContext
    inst = [W.batch_instance(s, max_cols=16, max_cells=8, n_range=(2, 5)) for s in range(6)]
    bc = BatchContext(inst)
    f = bc.forcing()
    g = bc.inflow()
    u, infos = bc.solve(f, g, rtol=1e-11, restart=30, max_it=3000)
    parts = bc.split(u.cpu().numpy())
    assert all(i["converged"] for i in infos), [i["res_f"] / i["rhs_norm"] for i in infos]
    for (mesh, spec), ub in zip(inst, parts):
        prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
        uh, conv, _ = prob.solve(mesh, ksp_type="gmres", rtol=1e-12, x0="zero")
        ref = uh.to_vector()
        assert np.linalg.norm(ub - ref) <= 1e-8 * np.linalg.norm(ref)


def test_batched_repeat_is_stable():
    """A second solve on the same handle replays the captured cycle graph."""
    from rtg import workloads as W
    from rtg.batch import BatchContext
    inst = [W.batch_instance(s, max_cols=12, max_cells=6, n_range=(2, 4)) for s in range(10, 14)]
    bc = BatchContext(inst)
    f = bc.forcing()
    g = bc.inflow()
    u1, i1 = bc.solve(f, g, rtol=1e-10)
    u2, i2 = bc.solve(f, g, rtol=1e-10)
    d = (u1 - u2).norm().item() / u1.norm().item()
    assert d < 1e-12 and all(i["converged"] for i in i2)


def test_batched_matches_oracle():
    """Five instances of the batched family (degrees 1, 3, 4, 6 and 7; 7 to 13
    columns; 5 to 8 angular cells) solved in one batch, each checked against
    the CPU oracle's solve of the reference's assembled system (scipy GMRES
    with the oracle sweep to 1e-13) in the quadrature-weighted L2 norm."""
    from oracle import rt_oracle as O
    from rtg import workloads as W
    from rtg.batch import BatchContext
    seeds = (42, 51, 46, 53, 55)
    inst = [W.batch_instance(s, max_cols=12, max_cells=8, n_range=(2, 8)) for s in seeds]
    bc = BatchContext(inst)
    u, infos = bc.solve(bc.forcing(), bc.inflow(), rtol=1e-11, restart=30, max_it=3000)
    assert all(i["converged"] for i in infos)
    for (mesh, spec), ub in zip(inst, bc.split(u.cpu().numpy())):
        o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
        ref, _, info = O.solve_sweep_gmres(o, o["layout"], rtol=1e-13, maxiter=400)
        assert info == 0
        w = O.l2_weights(mesh, o["layout"])
        err = np.sqrt(np.sum(w * (ub - ref) ** 2) / np.sum(w * ref ** 2))
        assert err < 1e-9, (mesh.get_ndof(), err)

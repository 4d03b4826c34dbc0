"""Pin the CPU oracle against the reference's own outputs (golden fixtures)."""
import numpy as np
import pytest
import scipy.sparse as sp

import golden_io
from oracle import rt_oracle as O


def test_quadrature_matches_reference():
    z = np.load(golden_io.GOLDEN + "/quadrature.npz")
    for n in range(1, 13):
        x, w = O.lgl_nodes(n)
        np.testing.assert_allclose(x, z["lgl_x_%d" % n], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, z["lgl_w_%d" % n], rtol=1e-14, atol=0)
        x, w = O.lg_nodes(n)
        np.testing.assert_allclose(x, z["lg_x_%d" % n], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, z["lg_w_%d" % n], rtol=1e-14, atol=0)


def _close(A, B, rtol=1e-13):
    D = (A - B).tocsr()
    scale = abs(B).max()
    assert abs(D).max() <= rtol * scale, (abs(D).max(), scale)
    # same sparsity up to entries that sit at the drop threshold
    pa = set(zip(*A.nonzero()))
    pb = set(zip(*B.nonzero()))
    assert len(pa ^ pb) <= max(2, 1e-4 * len(pb))


@pytest.fixture(scope="module", params=golden_io.CASES)
def case(request):
    name = request.param
    g = golden_io.load(name)
    mesh_fn, prob_fn = golden_io.problem(name)
    spec = prob_fn()
    mesh = mesh_fn()
    o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    return name, g, o, spec


def test_blocks(case):
    name, g, o, _ = case
    for nm in ("M", "S", "MS", "IC", "BC"):
        _close(o[nm], g[nm])


def test_vectors_and_mask(case):
    name, g, o, _ = case
    np.testing.assert_array_equal(o["mask"], g["mask"])
    np.testing.assert_allclose(o["f"], g["f"], rtol=1e-13, atol=1e-15 * abs(g["f"]).max())
    np.testing.assert_allclose(o["g"], g["g"], rtol=1e-13, atol=1e-15 * abs(g["g"]).max())


def test_direct_solution(case):
    name, g, o, _ = case
    u = O.solve_direct(o["A"], o["f"], o["g"], o["mask"])
    err = np.linalg.norm(u - g["u"]) / np.linalg.norm(g["u"])
    assert err < 1e-11, err


def test_manufactured_error_cfg1():
    g = golden_io.load("cfg1")
    mesh_fn, prob_fn = golden_io.problem("cfg1")
    spec = prob_fn()
    mesh = mesh_fn()
    X, Y, T = O.node_coords(mesh)
    w = O.l2_weights(mesh)
    ue = spec.u_exact(X, Y, T)
    err = np.sqrt(np.sum(w * (g["u"] - ue) ** 2) / np.sum(w * ue ** 2))
    np.testing.assert_allclose(err, float(g["rel_l2_err_exact"]), rtol=1e-10)


@pytest.mark.parametrize("name", ["cfg1", "small_random", "hp_hanging"])
def test_oracle_sweep_gmres_reaches_reference_solution(name):
    g = golden_io.load(name)
    mesh_fn, prob_fn = golden_io.problem(name)
    spec = prob_fn()
    o = O.assemble(mesh_fn(), spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    u, its, info = O.solve_sweep_gmres(o, o["layout"], rtol=1e-12)
    assert info == 0 and its < 40
    assert np.linalg.norm(u - g["u"]) / np.linalg.norm(g["u"]) < 1e-10

"""librtg's error indicators and hp steering (rtg.ErrorIndicator) against the
reference's own outputs (golden fixtures of tests/golden/make_golden_amr.py)
and against the CPU oracle on a larger adaptive mesh."""
import os

import numpy as np
import pytest

import golden_io
from oracle import amr_oracle as AO

pytestmark = pytest.mark.gpu
FORMS = {"": 0, "h": 1, "p": 2}


def _golden(name):
    z = np.load(os.path.join(golden_io.GOLDEN, "amr_" + name + ".npz"))
    return {k: z[k] for k in z.files}


def _flat(ind, mesh):
    cols = sorted(mesh.cols.keys())
    c = ind.cols
    cells = [(k, kk) for k in cols for kk in sorted(mesh.cols[k].cells)]
    return {"col_err": np.array([c[k].error for k in cols]),
            "col_do_ref": np.array([c[k].do_ref for k in cols]),
            "col_form": np.array([FORMS[c[k].ref_form] for k in cols]),
            "cell_err": np.array([c[k].cells[kk].error for k, kk in cells]),
            "cell_do_ref": np.array([c[k].cells[kk].do_ref for k, kk in cells]),
            "cell_form": np.array([FORMS[c[k].cells[kk].ref_form] for k, kk in cells])}


@pytest.mark.parametrize("name", golden_io.CASES)
def test_indicators_match_reference(name):
    from rtg import ErrorIndicator, Projection
    g = _golden(name)
    mesh = golden_io.problem(name)[0]()
    proj = Projection(mesh)
    proj.from_vector(g["u"])
    tol = tuple(float(t) for t in g["ref_tol"])
    ind = ErrorIndicator(proj, "all", "hp", tol)
    ind.error_angular_jump()
    f = _flat(ind, mesh)
    np.testing.assert_allclose(f["col_err"], g["ang_col_err"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(f["cell_err"], g["ang_cell_err"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(ind.error, g["ang_error"], rtol=1e-12)
    np.testing.assert_allclose(ind.error_to_resolve, g["ang_error_to_resolve"], rtol=1e-12)
    for k in ("col_do_ref", "col_form", "cell_do_ref", "cell_form"):
        np.testing.assert_array_equal(f[k], g["ang_" + k], err_msg=k)
    ind.error_spatial_jump()
    f = _flat(ind, mesh)
    np.testing.assert_allclose(f["col_err"], g["spt_col_err"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(ind.error, g["spt_error"], rtol=1e-12)
    np.testing.assert_allclose(ind.error_to_resolve, g["spt_error_to_resolve"], rtol=1e-12)
    for k in ("col_do_ref", "col_form"):
        np.testing.assert_array_equal(f[k], g["spt_" + k], err_msg=k)
    cols = sorted(mesh.cols.keys())
    np.testing.assert_array_equal([FORMS[ind.col_hp_steer(k)] for k in cols], g["hp_col_form"])
    np.testing.assert_array_equal([FORMS[ind.cell_hp_steer(k, kk)] for k in cols for kk in sorted(mesh.cols[k].cells)],
                                  g["hp_cell_form"])
    ind.close()


def test_indicators_on_adaptive_mesh_match_oracle():
    """The 2.2e5-DOF adaptive workload with a seeded smooth field: squared jumps
    and lp estimates against the oracle, flags and forms identical."""
    from rtg import ErrorIndicator, Projection, workloads as W
    mesh = W.config2_mesh()
    rng = np.random.default_rng(3)
    a, b, c = rng.uniform(0.5, 2.0, 3)
    proj = Projection(mesh, lambda x, y, th: np.exp(-a * (x - 1.5) ** 2 - b * (y - 1.) ** 2) * (1. + 0.5 * np.cos(th - c)))
    u = np.asarray(proj.to_vector())
    ind = ErrorIndicator(proj, "all", "hp", (0.3, 0.3))
    ind.error_angular_jump()
    ref = AO.indicator(mesh, u, "ang", "all", "hp", (0.3, 0.3))
    cols = sorted(mesh.cols.keys())
    got = np.array([ind.cols[k].cells[kk].error for k in cols for kk in sorted(mesh.cols[k].cells)])
    want = np.array([ref["cols"][k]["cells"][kk]["error"] for k in cols for kk in sorted(mesh.cols[k].cells)])
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-14)
    assert [ind.cols[k].ref_form for k in cols] == [ref["cols"][k]["ref_form"] for k in cols]
    assert [ind.cols[k].cells[kk].do_ref for k in cols for kk in sorted(mesh.cols[k].cells)] == \
        [ref["cols"][k]["cells"][kk]["do_ref"] for k in cols for kk in sorted(mesh.cols[k].cells)]
    ind.error_spatial_jump()
    sp = AO.spatial_jump(mesh, u)
    np.testing.assert_allclose([ind.cols[k].error ** 2 for k in cols], [sp[k] for k in cols], rtol=1e-11, atol=1e-16)
    # lp = log(.. / a_top^2) / (2 log(n - 1)): the top Legendre coefficient of a
    # smooth field is a sum that cancels to ~1e-10 of its terms, so lp agrees to
    # ~1e-4 absolute (FP64 on both sides, different summation orders); the p/h
    # decisions must agree exactly
    V = AO.cell_vals(mesh, u)
    lp_col, lp_cell = ind._hp()
    want = np.array([AO.col_lp(mesh, u, k, V) for k in cols])
    np.testing.assert_allclose(np.array([lp_col[k] for k in cols]), want, rtol=0, atol=1e-3)
    cells = [(k, kk) for k in cols for kk in sorted(mesh.cols[k].cells)]
    want = np.array([AO.cell_lp(mesh, u, k, kk, V) for k, kk in cells])
    np.testing.assert_allclose(np.array([lp_cell[c] for c in cells]), want, rtol=0, atol=1e-3)
    assert [ind.col_hp_steer(k) for k in cols] == [AO.col_form(mesh, k, AO.col_lp(mesh, u, k, V)) for k in cols]
    assert [ind.cell_hp_steer(k, kk) for k, kk in cells] == \
        [AO.cell_form(mesh, k, kk, AO.cell_lp(mesh, u, k, kk, V)) for k, kk in cells]
    ind.close()


@pytest.mark.parametrize("field", ["zero", "constant"])
def test_indicators_edge_fields(field):
    """A zero field (every jump exactly 0 and every lp infinite: the top
    coefficients vanish): errors, flags and forms as the oracle's, including
    the threshold ties (0 >= tol * 0 flags everything).  A constant field:
    every jump zero to rounding (which cells pass a threshold set by rounding
    residue is not compared)."""
    from rtg import ErrorIndicator, Projection, workloads as W
    mesh = W.hanging_hp_mesh()
    proj = Projection(mesh, (lambda x, y, th: 0. * x) if field == "zero" else (lambda x, y, th: 0. * x + 2.5))
    u = np.asarray(proj.to_vector())
    for kind in ("ang", "spt"):
        ind = ErrorIndicator(proj, "all", "hp", (0.5, 0.5))
        (ind.error_angular_jump if kind == "ang" else ind.error_spatial_jump)()
        ref = AO.indicator(mesh, u, kind, "all", "hp", (0.5, 0.5))
        cols = sorted(mesh.cols.keys())
        assert ind.error == pytest.approx(ref["error"], abs=1e-13)
        if field == "constant":
            assert ind.error <= 1e-12
            ind.close()
            continue
        assert [ind.cols[k].do_ref for k in cols] == [ref["cols"][k]["do_ref"] for k in cols]
        assert [ind.cols[k].ref_form for k in cols] == [ref["cols"][k]["ref_form"] for k in cols]
        cells = [(k, kk) for k in cols for kk in sorted(mesh.cols[k].cells)]
        assert [ind.cols[k].cells[kk].do_ref for k, kk in cells] == [ref["cols"][k]["cells"][kk]["do_ref"]
                                                                      for k, kk in cells]
        assert [ind.cols[k].cells[kk].ref_form for k, kk in cells] == [ref["cols"][k]["cells"][kk]["ref_form"]
                                                                        for k, kk in cells]
        ind.close()

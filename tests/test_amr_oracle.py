"""Pin the AMR indicator oracle against the reference's own outputs
(tests/golden/make_golden_amr.py: error_angular_jump, error_spatial_jump,
col_hp_steer and cell_hp_steer run on each golden case's direct solution)."""
import os

import numpy as np
import pytest

import golden_io
from oracle import amr_oracle as AO

FORMS = {"": 0, "h": 1, "p": 2}


def _load(name):
    z = np.load(os.path.join(golden_io.GOLDEN, "amr_" + name + ".npz"))
    return {k: z[k] for k in z.files}


def _flatten(ind, mesh):
    cols = sorted(mesh.cols.keys())
    c = ind["cols"]
    out = {"col_err": np.array([c[k]["error"] for k in cols]),
           "col_do_ref": np.array([c[k]["do_ref"] for k in cols]),
           "col_form": np.array([FORMS[c[k]["ref_form"]] for k in cols]),
           "cell_err": np.array([c[k]["cells"][kk]["error"] for k in cols for kk in sorted(mesh.cols[k].cells)]),
           "cell_do_ref": np.array([c[k]["cells"][kk]["do_ref"] for k in cols for kk in sorted(mesh.cols[k].cells)]),
           "cell_form": np.array([FORMS[c[k]["cells"][kk]["ref_form"]] for k in cols
                                  for kk in sorted(mesh.cols[k].cells)])}
    return out


@pytest.mark.parametrize("name", golden_io.CASES)
def test_angular_jump_matches_reference(name):
    g = _load(name)
    mesh = golden_io.problem(name)[0]()
    ind = AO.indicator(mesh, g["u"], "ang", "all", "hp", tuple(g["ref_tol"]))
    f = _flatten(ind, mesh)
    np.testing.assert_allclose(f["col_err"], g["ang_col_err"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(f["cell_err"], g["ang_cell_err"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(ind["error"], g["ang_error"], rtol=1e-12)
    np.testing.assert_allclose(ind["error_to_resolve"], g["ang_error_to_resolve"], rtol=1e-12)
    assert ind["col_max_error"] == pytest.approx(float(g["ang_col_max"]), rel=1e-12)
    assert ind["cell_max_error"] == pytest.approx(float(g["ang_cell_max"]), rel=1e-12)
    for k in ("col_do_ref", "col_form", "cell_do_ref", "cell_form"):
        np.testing.assert_array_equal(f[k], g["ang_" + k], err_msg=k)


@pytest.mark.parametrize("name", golden_io.CASES)
def test_spatial_jump_matches_reference(name):
    g = _load(name)
    mesh = golden_io.problem(name)[0]()
    ind = AO.indicator(mesh, g["u"], "spt", "all", "hp", tuple(g["ref_tol"]))
    f = _flatten(ind, mesh)
    np.testing.assert_allclose(f["col_err"], g["spt_col_err"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(ind["error"], g["spt_error"], rtol=1e-12)
    assert ind["col_max_error"] == pytest.approx(float(g["spt_col_max"]), rel=1e-12)
    # cells carry -INF (INF = the largest float): none is flagged
    assert ind["cell_max_error"] == float(g["spt_cell_max"]) == -np.finfo(np.float64).max
    np.testing.assert_allclose(ind["error_to_resolve"], g["spt_error_to_resolve"], rtol=1e-12)
    for k in ("col_do_ref", "col_form"):
        np.testing.assert_array_equal(f[k], g["spt_" + k], err_msg=k)


@pytest.mark.parametrize("name", golden_io.CASES)
def test_hp_steering_matches_reference(name):
    g = _load(name)
    mesh = golden_io.problem(name)[0]()
    V = AO.cell_vals(mesh, g["u"])
    cols = sorted(mesh.cols.keys())
    cf = [FORMS[AO.col_form(mesh, k, AO.col_lp(mesh, g["u"], k, V))] for k in cols]
    ef = [FORMS[AO.cell_form(mesh, k, kk, AO.cell_lp(mesh, g["u"], k, kk, V))]
          for k in cols for kk in sorted(mesh.cols[k].cells)]
    np.testing.assert_array_equal(cf, g["hp_col_form"])
    np.testing.assert_array_equal(ef, g["hp_cell_form"])

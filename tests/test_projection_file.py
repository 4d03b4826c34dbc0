"""Projection files: rtg.Projection writes and reads the bytes the reference's
Projection.to_file writes (dg/projection/to_file.py:10-19: mesh JSON plus the
global-order vector as raw float64) and from_file reads
(dg/projection/from_file.py:14-21).  The fixture was written by the
reference itself (tests/golden/make_golden.py, write_projection_fixture)."""
import json
import os

import numpy as np

import golden_io
from rtg import mesh as rmesh
from rtg import projection as rproj
from rtg import workloads as W


def _fixture():
    z = np.load(os.path.join(golden_io.GOLDEN, "projection_file.npz"))
    return str(z["mesh_json"]), z["proj_bytes"].tobytes()


def _func(x, y, th):
    # the function the fixture sampled (make_golden.projection_func)
    return np.sin(1.3 * x + 0.4) * np.cos(0.7 * y) * (1. + 0.25 * np.sin(2. * th)) + 0.1 * th


def test_to_file_is_byte_identical(tmp_path):
    mesh_json, raw = _fixture()
    proj = rproj.Projection(W.small_random_mesh(), _func)
    pf, mf = tmp_path / "projection.npy", tmp_path / "mesh.json"
    proj.to_file(str(pf), write_mesh=True, mesh_file_path=str(mf))
    assert pf.read_bytes() == raw
    assert json.loads(mf.read_text()) == json.loads(mesh_json)


def test_from_file_reads_reference_files(tmp_path):
    mesh_json, raw = _fixture()
    pf, mf = tmp_path / "projection.npy", tmp_path / "mesh.json"
    pf.write_bytes(raw)
    mf.write_text(mesh_json)
    proj = rproj.from_file(str(mf), str(pf))
    np.testing.assert_array_equal(proj.to_vector(), np.frombuffer(raw, dtype=np.float64))
    assert rmesh.mesh_to_dict(proj.mesh) == json.loads(mesh_json)
    # and back out again, byte for byte
    out = tmp_path / "again.npy"
    proj.to_file(str(out), write_mesh=False)
    assert out.read_bytes() == raw


def test_dirac_branch_follows_truthiness():
    """A lone Dirac coordinate of 0.0 does not select the point-source branch
    (the reference tests any(dirac)); with another nonzero coordinate it is a
    real position (rt/boundary_conditions_vector.py:142-196)."""
    from oracle import rt_oracle as O
    from rtg.layout import MeshLayout
    from rtg.problem import _dirac_inflow
    mesh = W.small_random_mesh()
    spec = W.point_inflow_problem()
    bcs = spec.bcs_dirac[0]
    plain = O.boundary_conditions_vector(mesh, [bcs, [None, None, None]])
    zero_only = O.boundary_conditions_vector(mesh, [bcs, [0.0, None, None]])
    np.testing.assert_array_equal(zero_only, plain)
    lay = MeshLayout(mesh)
    for dirac in ([0.0, None, 0.3], [1.1, 0.5, None], [None, None, 2.0]):
        ref = O.boundary_conditions_vector(mesh, [bcs, dirac])
        np.testing.assert_allclose(_dirac_inflow(lay, bcs, dirac), ref, rtol=1e-14, atol=0.)

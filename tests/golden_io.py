"""Loading helpers for the golden fixtures made by tests/golden/make_golden.py."""
import json
import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["cfg1", "hp_hanging", "quad_none", "periodic", "small_random", "dirac"]


def load(case):
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    out = {k: z[k] for k in z.files}
    N = len(out["f"])
    for nm in ("S", "MS", "IC", "BC"):
        out[nm] = sp.csr_matrix((out.pop(nm + "_data"), out.pop(nm + "_indices"),
                                 out.pop(nm + "_indptr")), shape=(N, N))
    out["M"] = sp.diags(out["M_diag"], format="csr")
    out["A"] = ((out["BC"] - out["IC"]) + out["MS"]).tocsr()
    out["mesh_dict"] = json.loads(str(out["mesh_json"]))
    return out


def problem(case):
    from rtg import workloads as W
    return {
        "cfg1": (W.config1_mesh, lambda: W.manufactured_problem()),
        "hp_hanging": (W.hanging_hp_mesh, lambda: W.smooth_variable_problem(1., 2.)),
        "quad_none": (W.quadrant_free_mesh, lambda: W.smooth_variable_problem(1., 1., g=0.3)),
        "periodic": (W.periodic_mesh, lambda: W.smooth_variable_problem(1., 1., g=0.5)),
        "small_random": (W.small_random_mesh, lambda: W.gaussian_bump_problem()),
        "dirac": (W.small_random_mesh, lambda: W.point_inflow_problem()),
    }[case]

"""Generate golden fixtures for the AMR error indicators from the reference.

Run in a container where the reference source tree is present:

    python tests/golden/make_golden_amr.py --ref <reference checkout>

(``--ref`` may also come from the environment variable RT_REFERENCE.)

For every golden case of make_golden.py (which must have been run first: its
``<case>.npz`` holds the reference mesh and the reference direct solution u),
this builds the reference ``Projection`` from u and runs the reference's own
indicator code on it: ``error_angular_jump``, ``error_spatial_jump``,
``col_hp_steer`` and ``cell_hp_steer`` (src/amr/Error_Indicator).  The
package's ``__init__`` cannot be imported as shipped (``ref_by_ind.py``
imports ``..error_indicator``, which does not exist), so the four modules are
loaded directly and attached to a minimal stand-in of ``Error_Indicator``
whose ``__init__`` copies the reference's (class_Error_Indicator.py:12-20).
Every method that runs is the reference's.

Each case writes ``tests/golden/amr_<case>.npz``: with ref_kind "all",
ref_form "hp", ref_tol [0.5, 0.5], for the angular jump the cell and column
errors, the maxima, the mesh error, error_to_resolve and every column's and
cell's do_ref and ref_form; for the spatial jump the same at column level; and
col_hp_steer / cell_hp_steer on every column and cell.  Forms are coded
'' = 0, 'h' = 1, 'p' = 2.
"""

import argparse
import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

FORMS = {"": 0, "h": 1, "p": 2}
TOL = [0.5, 0.5]


def load_reference_indicator(src):
    for name, path in (("amr", "amr"), ("amr.Error_Indicator", "amr/Error_Indicator"),
                       ("amr.Error_Indicator.error", "amr/Error_Indicator/error")):
        m = types.ModuleType(name)
        m.__path__ = [os.path.join(src, path)]
        sys.modules[name] = m
    aj = importlib.import_module("amr.Error_Indicator.error.error_angular_jump").error_angular_jump
    sj = importlib.import_module("amr.Error_Indicator.error.error_spatial_jump").error_spatial_jump
    ch = importlib.import_module("amr.Error_Indicator.col_hp_steer").col_hp_steer
    eh = importlib.import_module("amr.Error_Indicator.cell_hp_steer").cell_hp_steer
    import consts

    class RefIndicator:
        def __init__(self, proj, ref_kind="all", ref_form="hp", ref_tol=[consts.INF, consts.INF]):
            self.proj = proj
            self.ref_kind = ref_kind
            self.ref_form = ref_form
            [self.ang_ref_tol, self.spt_ref_tol] = ref_tol

        error_angular_jump = aj
        error_spatial_jump = sj
        col_hp_steer = ch
        cell_hp_steer = eh

    return RefIndicator


def record(ind, prefix, cells_too):
    cols = sorted(ind.cols.keys())
    out = {prefix + "col_err": np.array([ind.cols[k].error for k in cols]),
           prefix + "col_do_ref": np.array([bool(ind.cols[k].do_ref) for k in cols]),
           prefix + "col_form": np.array([FORMS[ind.cols[k].ref_form] for k in cols], dtype=np.int8),
           prefix + "error": np.array(ind.error), prefix + "col_max": np.array(ind.col_max_error),
           prefix + "cell_max": np.array(ind.cell_max_error),
           prefix + "error_to_resolve": np.array(ind.error_to_resolve)}
    if cells_too:
        ce, cd, cf = [], [], []
        for k in cols:
            for kk in sorted(ind.cols[k].cells.keys()):
                c = ind.cols[k].cells[kk]
                ce.append(c.error)
                cd.append(bool(getattr(c, "do_ref", False)))
                cf.append(FORMS[getattr(c, "ref_form", "")])
        out.update({prefix + "cell_err": np.array(ce), prefix + "cell_do_ref": np.array(cd),
                    prefix + "cell_form": np.array(cf, dtype=np.int8)})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("RT_REFERENCE"),
                    help="root of the reference checkout (its src/ is imported)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("--ref (or RT_REFERENCE) must name the reference checkout")
    MG.install_stubs()
    src = os.path.join(args.ref, "src")
    sys.path.insert(0, src)
    from dg.mesh import Mesh as RefMesh
    from dg.projection import Projection as RefProjection
    RefIndicator = load_reference_indicator(src)
    import warnings
    warnings.simplefilter("ignore", RuntimeWarning)   # log(nx - 1) = 0 at nx = 2: the reference divides by it
    for name, (mesh_fn, _) in MG.cases().items():
        g = np.load(os.path.join(HERE, name + ".npz"))
        mesh = mesh_fn(mesh_cls=RefMesh)
        proj = RefProjection(mesh)
        proj.from_vector(np.array(g["u"]))
        out = {"u": np.array(g["u"]), "ref_tol": np.array(TOL)}
        ind = RefIndicator(proj, "all", "hp", TOL)
        ind.error_angular_jump()
        out.update(record(ind, "ang_", True))
        ind = RefIndicator(proj, "all", "hp", TOL)
        ind.error_spatial_jump()
        out.update(record(ind, "spt_", False))
        ind = RefIndicator(proj, "all", "hp", TOL)
        cols = sorted(proj.cols.keys())
        out["hp_col_form"] = np.array([FORMS[ind.col_hp_steer(k)] for k in cols], dtype=np.int8)
        out["hp_cell_form"] = np.array([FORMS[ind.cell_hp_steer(k, kk)] for k in cols
                                        for kk in sorted(proj.cols[k].cells.keys())], dtype=np.int8)
        np.savez_compressed(os.path.join(HERE, "amr_" + name + ".npz"), **out)
        print("{:14s} ang error {:.6e}  spatial error {:.6e}  hp p-columns {}/{}  p-cells {}/{}".format(
            name, float(out["ang_error"]), float(out["spt_error"]), int((out["hp_col_form"] == 2).sum()),
            len(cols), int((out["hp_cell_form"] == 2).sum()), len(out["hp_cell_form"])))


if __name__ == "__main__":
    main()

"""Generate golden fixtures for the RT solve from the reference itself.

Run in a container where the reference source tree is present:

    python tests/golden/make_golden.py --ref <reference checkout> [--only CASE]

(``--ref`` may also come from the environment variable RT_REFERENCE.)

The reference's ``src/rt`` modules import petsc4py and mpi4py at module level.
Neither is installed here, so two stub modules stand in (identity ``bcast``,
no-op ``Barrier``, rank 0 of 1).  With them, the reference's per-column
builders -- ``mass_matrix.calc_col_matrix``, ``scattering_matrix.calc_col_matrix``,
``preconditioner_matrix.calc_col_matrix``, ``interior_convection_matrix.calc_col_matrix``,
``boundary_convection_matrix.calc_col_matrix``, ``forcing_vector.calc_col_vec``,
``boundary_conditions_vector.calc_col_vec`` -- run unchanged.  They are
assembled exactly as the PETSc wrappers place them (column blocks on the
diagonal, boundary-convection column blocks by ``sp.bmat``:
rt/boundary_convection_matrix.py:57-105) and the split system of
rt/solve.py:81-101 is solved directly with ``scipy.sparse.linalg.spsolve``.

Each case writes ``tests/golden/<case>.npz`` holding the reference mesh (JSON
of dg/mesh/to_file.py), the blocks M (diagonal), S, MS, IC, BC (CSR), the
vectors f, g, the interior mask and the direct solution u.  The ``dirac`` case
takes its inflow data through the reference's point-source branch
(rt/boundary_conditions_vector.py:142-196).

``projection_file.npz`` holds what the reference's ``Projection.to_file``
writes (dg/projection/to_file.py:10-19) for a sampled function on the
``small_random`` mesh: the mesh JSON text and the raw float64 bytes.
"""

import argparse
import json
import os
import sys
import types

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.normpath(os.path.join(HERE, os.pardir, os.pardir))
sys.path.insert(0, os.path.join(REPO, "radiative-transfer-amr_gb300"))


def install_stubs():
    mpi4py = types.ModuleType("mpi4py")
    MPI = types.ModuleType("mpi4py.MPI")

    class Comm:
        def bcast(self, x, root=0):
            return x

        def Barrier(self):
            pass

        def barrier(self):
            pass

        def gather(self, x, root=0):
            return [x]

    MPI.COMM_WORLD = Comm()
    MPI.Intracomm = Comm
    mpi4py.MPI = MPI
    petsc4py = types.ModuleType("petsc4py")
    PETSc = types.ModuleType("petsc4py.PETSc")

    class Sys:
        @staticmethod
        def isInitialized():
            return True

        @staticmethod
        def Print(*a):
            print(*a)

    class PComm:
        def getRank(self):
            return 0

        def getSize(self):
            return 1

    PETSc.Sys = Sys
    PETSc.COMM_WORLD = PComm()
    PETSc.Comm = PComm
    for n in ("Mat", "Vec", "KSP", "PC", "IS"):
        setattr(PETSc, n, type(n, (object,), {}))
    petsc4py.PETSc = PETSc
    petsc4py.init = lambda *a, **k: None
    sys.modules.update({"mpi4py": mpi4py, "mpi4py.MPI": MPI,
                        "petsc4py": petsc4py, "petsc4py.PETSc": PETSc})


def ref_assemble(mesh, spec):
    import rt.mass_matrix as mm
    import rt.scattering_matrix as sm
    import rt.preconditioner_matrix as pm
    import rt.interior_convection_matrix as icm
    import rt.boundary_convection_matrix as bcm
    import rt.forcing_vector as fv
    import rt.boundary_conditions_vector as bv
    from dg.matrix import get_intr_mask, get_col_idxs

    keys = sorted(mesh.cols.keys())
    M = sp.block_diag([mm.calc_col_matrix(mesh, k, spec.kappa) for k in keys], format="csr")
    S = sp.block_diag([sm.calc_col_matrix(mesh, k, spec.sigma, spec.Phi) for k in keys],
                      format="csr")
    MS = sp.block_diag([pm.calc_col_matrix(mesh, k, spec.kappa, spec.sigma, spec.Phi)[0]
                        for k in keys], format="csr")
    IC = sp.block_diag([icm.calc_col_matrix(mesh, k) for k in keys], format="csr")

    # rt/boundary_convection_matrix.py:57-105 (root-rank assembly)
    ncols, col_idxs = get_col_idxs(mesh)
    blocks = [[None] * ncols for _ in range(ncols)]
    for k0 in keys:
        c0 = col_idxs[k0]
        for F in range(4):
            m00, (k1, m01), (k2, m02) = bcm.calc_col_matrix(mesh, k0, F)
            blocks[c0][c0] = m00 if blocks[c0][c0] is None else blocks[c0][c0] + m00
            if k1 is not None:
                c1 = col_idxs[k1]
                blocks[c0][c1] = m01 if blocks[c0][c1] is None else blocks[c0][c1] + m01
            if k2 is not None:
                c2 = col_idxs[k2]
                blocks[c0][c2] = m02 if blocks[c0][c2] is None else blocks[c0][c2] + m02
    BC = sp.bmat(blocks, format="csr")

    f = np.concatenate([fv.calc_col_vec(mesh, k, spec.f) for k in keys])
    g = np.concatenate([bv.calc_col_vec(mesh, k, spec.bcs_dirac) for k in keys])
    mask = np.asarray(get_intr_mask(mesh), dtype=bool)
    return M, S, MS, IC, BC, f, g, mask


def direct_solve(A, f, g, mask):
    I = np.nonzero(mask)[0]
    B = np.nonzero(~mask)[0]
    A = A.tocsr()
    rhs = f[I] - A[I][:, B] @ g[B]
    u = np.zeros(len(mask))
    u[I] = spla.spsolve(A[I][:, I].tocsc(), rhs)
    u[B] = g[B]
    return u


def node_coords(mesh):
    from dg.quadrature import quad_xyth
    from dg.projection import push_forward
    X, Y, T = [], [], []
    for ck in sorted(mesh.cols.keys()):
        col = mesh.cols[ck]
        nx, ny = col.ndofs
        xxb, _, yyb, _, _, _ = quad_xyth(nnodes_x=nx, nnodes_y=ny)
        xx = push_forward(col.pos[0], col.pos[2], xxb)
        yy = push_forward(col.pos[1], col.pos[3], yyb)
        for kk in sorted(col.cells.keys()):
            cell = col.cells[kk]
            nth = cell.ndofs[0]
            _, _, _, _, tb, _ = quad_xyth(nnodes_th=nth)
            th = push_forward(cell.pos[0], cell.pos[1], tb)
            X.append(np.broadcast_to(xx[:, None, None], (nx, ny, nth)).ravel())
            Y.append(np.broadcast_to(yy[None, :, None], (nx, ny, nth)).ravel())
            T.append(np.broadcast_to(th[None, None, :], (nx, ny, nth)).ravel())
    return np.concatenate(X), np.concatenate(Y), np.concatenate(T)


def csr_fields(name, A):
    A = A.tocsr()
    A.sort_indices()
    return {name + "_data": A.data, name + "_indices": A.indices.astype(np.int32),
            name + "_indptr": A.indptr.astype(np.int64)}


def cases():
    from rtg import workloads as W
    return {
        "cfg1": (W.config1_mesh, lambda: W.manufactured_problem()),
        "hp_hanging": (W.hanging_hp_mesh, lambda: W.smooth_variable_problem(1., 2.)),
        "quad_none": (W.quadrant_free_mesh, lambda: W.smooth_variable_problem(1., 1., g=0.3)),
        "periodic": (W.periodic_mesh, lambda: W.smooth_variable_problem(1., 1., g=0.5)),
        "small_random": (W.small_random_mesh, lambda: W.gaussian_bump_problem()),
        "dirac": (W.small_random_mesh, lambda: W.point_inflow_problem()),
    }


def projection_func(x, y, th):
    """The function sampled for the projection-file fixture."""
    return np.sin(1.3 * x + 0.4) * np.cos(0.7 * y) * (1. + 0.25 * np.sin(2. * th)) + 0.1 * th


def write_projection_fixture(RefMesh):
    from rtg import workloads as W
    from dg.projection import Projection as RefProjection
    mesh = W.small_random_mesh(mesh_cls=RefMesh)
    proj = RefProjection(mesh, projection_func)
    pf = os.path.join(HERE, "_proj_tmp.npy")
    mf = os.path.join(HERE, "_proj_mesh_tmp.json")
    proj.to_file(pf, write_mesh=True, mesh_file_path=mf)
    with open(pf, "rb") as fh:
        raw = fh.read()
    with open(mf) as fh:
        mesh_json = fh.read()
    os.remove(pf)
    os.remove(mf)
    np.savez_compressed(os.path.join(HERE, "projection_file.npz"), mesh_json=np.array(mesh_json),
                        proj_bytes=np.frombuffer(raw, dtype=np.uint8))
    print("projection_file  {} bytes of float64".format(len(raw)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("RT_REFERENCE"),
                    help="root of the reference checkout (its src/ is imported)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if not args.ref:
        ap.error("--ref (or RT_REFERENCE) must name the reference checkout")
    install_stubs()
    sys.path.insert(0, os.path.join(args.ref, "src"))
    from dg.mesh import Mesh as RefMesh
    from dg.quadrature import quad_xyth

    # quadrature pins: nodes/weights for n = 1..12
    q = {}
    for n in range(1, 13):
        xb, wx, _, _, tb, wt = quad_xyth(nnodes_x=n, nnodes_th=n)
        q["lgl_x_%d" % n] = np.asarray(xb, dtype=np.float64)
        q["lgl_w_%d" % n] = np.asarray(wx, dtype=np.float64)
        q["lg_x_%d" % n] = np.asarray(tb, dtype=np.float64)
        q["lg_w_%d" % n] = np.asarray(wt, dtype=np.float64)
    if args.only is None:
        np.savez_compressed(os.path.join(HERE, "quadrature.npz"), **q)
    if args.only in (None, "projection_file"):
        write_projection_fixture(RefMesh)

    for name, (mesh_fn, prob_fn) in cases().items():
        if args.only and name != args.only:
            continue
        mesh = mesh_fn(mesh_cls=RefMesh)
        spec = prob_fn()
        M, S, MS, IC, BC, f, g, mask = ref_assemble(mesh, spec)
        A = (BC - IC) + MS
        u = direct_solve(A, f, g, mask)
        tmp = os.path.join(HERE, "_mesh_tmp.json")
        mesh.to_file(tmp)
        with open(tmp) as fh:
            mesh_json = fh.read()
        os.remove(tmp)
        out = {"mesh_json": np.array(mesh_json), "M_diag": M.diagonal(),
               "f": f, "g": g, "mask": mask, "u": u}
        for nm, mat in (("S", S), ("MS", MS), ("IC", IC), ("BC", BC)):
            out.update(csr_fields(nm, mat))
        if spec.u_exact is not None:
            X, Y, T = node_coords(mesh)
            ue = spec.u_exact(X, Y, T)
            w = M.diagonal() / (spec.kappa(X, Y) + 0. * X)
            err = np.sqrt(np.sum(w * (u - ue) ** 2) / np.sum(w * ue ** 2))
            out["rel_l2_err_exact"] = np.array(err)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("{:14s} N={:6d} interior={:6d} nnz(A)={:8d} size={:.2f} MB".format(
            name, len(f), int(mask.sum()), A.nnz,
            os.path.getsize(os.path.join(HERE, name + ".npz")) / 1e6),
            ("rel_l2_err_exact=%.4e" % out["rel_l2_err_exact"]) if "rel_l2_err_exact" in out else "")


if __name__ == "__main__":
    main()

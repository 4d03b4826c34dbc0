"""Nodal function on the hp mesh: the solution container returned by solve.

Mirrors dg/projection/class_Projection.py:17-97: ``Projection(mesh, func)``
samples func(x, y, th) at the nodes; ``cols[col_key].cells[cell_key].vals`` is
an [nx, ny, nth] array; ``to_vector``/``from_vector`` use the global DOF order
(dg/projection/to_vector.py:11-44, from_vector.py:11-40); ``to_file`` writes the
vector as raw float64 plus the mesh JSON (dg/projection/to_file.py:10-19)."""

import copy

import numpy as np

from .layout import MeshLayout, _eval
from . import mesh as _mesh


class ProjectionCell:
    def __init__(self, cell, vals):
        self.pos = cell.pos
        self.idx = cell.idx
        self.lv = cell.lv
        self.key = cell.key
        self.is_lf = cell.is_lf
        self.ndofs = cell.ndofs
        self.quadrant = cell.quadrant
        self.vals = vals

    def __eq__(self, other):
        return (self.key == other.key and self.ndofs == other.ndofs
                and np.array_equal(self.vals, other.vals))


class ProjectionColumn:
    def __init__(self, col, cells):
        self.pos = col.pos
        self.idx = col.idx
        self.lv = col.lv
        self.key = col.key
        self.is_lf = col.is_lf
        self.ndofs = col.ndofs
        self.nhbr_keys = col.nhbr_keys
        self.cells = cells

    def __eq__(self, other):
        return self.key == other.key and self.cells == other.cells


class Projection:
    def __init__(self, mesh, func=None):
        self.mesh = copy.deepcopy(mesh)
        self.Ls = self.mesh.Ls
        self.pbcs = self.mesh.pbcs
        self.has_th = self.mesh.has_th
        lay = MeshLayout(self.mesh)
        if func is None:
            vec = np.zeros(lay.N)
        else:
            X, Y, T = lay.node_coords()
            if self.mesh.has_th:
                vec = np.array(_eval(func, X, Y, T), dtype=np.float64)
            else:
                vec = np.array(_eval(lambda x, y, th: func(x, y), X, Y, T), dtype=np.float64)
        self._build(lay, vec)

    def _build(self, lay, vec):
        self.cols = {}
        for ci, ck in enumerate(lay.col_keys):
            col = self.mesh.cols[ck]
            nx, ny = col.ndofs[0], col.ndofs[1]
            cells = {}
            for e in range(int(lay.col_elem_start[ci]), int(lay.col_elem_start[ci + 1])):
                kk = lay.elem_keys[e][1]
                cell = col.cells[kk]
                o = int(lay.elem_off[e])
                n = nx * ny * cell.ndofs[0]
                cells[kk] = ProjectionCell(cell, np.array(vec[o:o + n]).reshape(nx, ny, cell.ndofs[0]))
            self.cols[ck] = ProjectionColumn(col, cells)

    def to_vector(self):
        out = []
        for ck in sorted(self.cols.keys()):
            col = self.cols[ck]
            for kk in sorted(col.cells.keys()):
                out.append(col.cells[kk].vals.reshape(-1))
        return np.concatenate(out)

    def from_vector(self, vec):
        self._build(MeshLayout(self.mesh), np.asarray(vec, dtype=np.float64))
        return self

    def to_file(self, file_path="projection.npy", write_mesh=True, mesh_file_path="mesh.json"):
        if write_mesh:
            self.mesh.to_file(mesh_file_path)
        self.to_vector().tofile(file_path)

    def __eq__(self, other):
        return self.mesh == other.mesh and self.cols == other.cols


def from_file(mesh_file_path="mesh.json", projection_file_path="projection.npy"):
    """dg/projection/from_file.py:14-21"""
    mesh = _mesh.from_file(mesh_file_path)
    proj = Projection(mesh, None)
    proj.from_vector(np.fromfile(projection_file_path))
    return proj

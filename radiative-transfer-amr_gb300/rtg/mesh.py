"""hp-mesh of the steady RT solve: a quadtree of spatial columns, each holding a
binary tree of angular cells.

This module is the host-side mesh the GPU solve consumes.  It keeps the object
model, keys, neighbour bookkeeping, refinement order and JSON layout of the
reference's ``dg.mesh`` package so that a mesh built here and a mesh built by
the reference are interchangeable (every function in ``rtg.layout`` reads only
the attributes listed below, so a reference ``Mesh`` object also works):

  Column: pos [x0, y0, x1, y1], idx [i0, i1], lv, key, is_lf, ndofs [nx, ny],
          cells {key: Cell}, nhbr_keys [[k, k] per face F = 0 right, 1 top,
          2 left, 3 bottom]                      (dg/mesh/column/class_Column.py:10-26)
  Cell:   pos [th0, th1], idx, lv, key, is_lf, ndofs [nth], quadrant (0..3 or
          None), nhbr_keys [k-, k+]               (dg/mesh/column/cell/class_Cell.py:11-25)

Only leaves are stored: refining a column or cell replaces it by its children
(dg/mesh/ref_col_spt.py:221, dg/mesh/ref_cell.py:405).
"""

import copy
import json
import math

PI = math.pi


def col_key_of(idx, lv):
    """Column key: sum_{l<lv} 4^l + 2^lv * idx[1] + idx[0] (dg/mesh/column/calc_key.py:9-17)."""
    base = 0
    for ll in range(lv):
        base += 4 ** ll
    return base + (2 ** lv) * idx[1] + idx[0]


def cell_key_of(idx, lv):
    """Cell key: sum_{l<lv} 2^l + idx (dg/mesh/column/cell/calc_key.py:9-17).

    A negative level contributes nothing (the parent lookup of a root cell asks
    for level -1 and gets key ``idx``)."""
    base = 0
    for ll in range(lv):
        base += 2 ** ll
    return base + idx


class Cell:
    """Angular cell [th0, th1] of one column (dg/mesh/column/cell/class_Cell.py:11-49)."""

    def __init__(self, pos, idx, lv, is_lf, ndofs, quadrant, nhbr_keys):
        self.pos = pos
        self.idx = idx
        self.lv = lv
        self.key = cell_key_of(idx, lv)
        self.is_lf = is_lf
        self.ndofs = ndofs
        self.quadrant = quadrant
        self.nhbr_keys = nhbr_keys

    def __eq__(self, other):
        return (self.pos == other.pos and self.idx == other.idx
                and self.lv == other.lv and self.key == other.key
                and self.is_lf == other.is_lf and self.ndofs == other.ndofs
                and self.quadrant == other.quadrant
                and self.nhbr_keys == other.nhbr_keys)

    def __repr__(self):
        return "Cell(key={}, lv={}, pos={}, ndofs={}, quadrant={})".format(
            self.key, self.lv, self.pos, self.ndofs, self.quadrant)


class Column:
    """Spatial column [x0,x1]x[y0,y1] with its angular cells
    (dg/mesh/column/class_Column.py:10-49)."""

    def __init__(self, pos, idx, lv, is_lf, ndofs, cells, nhbr_keys):
        self.pos = pos
        self.idx = idx
        self.lv = lv
        self.key = col_key_of(idx, lv)
        self.is_lf = is_lf
        self.ndofs = ndofs
        self.cells = cells
        self.nhbr_keys = nhbr_keys

    def add_cell(self, cell):
        self.cells[cell.key] = cell

    def del_cell(self, cell_key):
        del self.cells[cell_key]

    def nhbr_cell(self, cell_key, nhbr_loc="+"):
        """Leaf cell next to ``cell_key`` in angle, same level, parent level or
        child level, in that order (dg/mesh/column/nhbr_cell.py:13-63)."""
        cell = self.cells[cell_key]
        lv = cell.lv
        step = 1 if nhbr_loc == "+" else (-1 if nhbr_loc == "-" else 0)
        n_idx = (cell.idx + step) % (2 ** lv)
        cand = self.cells.get(cell_key_of(n_idx, lv))
        if cand is not None and cand.is_lf:
            return cand
        cand = self.cells.get(cell_key_of(math.floor(n_idx / 2), lv - 1))
        if cand is not None and cand.is_lf:
            return cand
        c_idx = 2 * n_idx if nhbr_loc == "+" else 2 * n_idx + 1
        cand = self.cells.get(cell_key_of(c_idx, lv + 1))
        if cand is not None and cand.is_lf:
            return cand
        return None

    def __eq__(self, other):
        return (self.pos == other.pos and self.idx == other.idx
                and self.lv == other.lv and self.key == other.key
                and self.is_lf == other.is_lf and self.ndofs == other.ndofs
                and self.cells == other.cells
                and self.nhbr_keys == other.nhbr_keys)

    def __repr__(self):
        return "Column(key={}, lv={}, pos={}, ndofs={}, ncells={})".format(
            self.key, self.lv, self.pos, self.ndofs, len(self.cells))


class Mesh:
    """Quadtree-in-space, binary-tree-in-angle hp mesh (dg/mesh/class_Mesh.py:12-90).

    ``Mesh(Ls, pbcs, ndofs=[nx, ny, nth], has_th)`` starts with one column over
    [0, Lx] x [0, Ly] holding one angular cell over [0, 2*pi]."""

    def __init__(self, Ls, pbcs, ndofs=(2, 2, 2), has_th=False):
        self.Ls = Ls
        self.pbcs = pbcs
        self.has_th = has_th
        if has_th:
            root_cell = Cell([0, 2 * PI], 0, 0, True, [ndofs[2]], None, [0, 0])
        else:
            root_cell = Cell([0, 0], 0, 0, True, [1], None, [None, None])
        nk = [[None, None], [None, None], [None, None], [None, None]]
        if pbcs[0]:
            nk[0] = [0, 0]
            nk[2] = [0, 0]
        if pbcs[1]:
            nk[1] = [0, 0]
            nk[3] = [0, 0]
        col = Column([0, 0, Ls[0], Ls[1]], [0, 0], 0, True, list(ndofs[0:2]),
                     {0: root_cell}, nk)
        self.cols = {col.key: col}

    # ------------------------------------------------------------------ basics
    def add_col(self, col):
        self.cols[col.key] = col

    def del_col(self, col_key):
        del self.cols[col_key]

    def get_ndof(self):
        """Total DOFs = sum over leaf elements of nx*ny*nth (dg/mesh/get_ndof.py:9-21)."""
        total = 0
        for col in self.cols.values():
            if not col.is_lf:
                continue
            nx, ny = col.ndofs[0], col.ndofs[1]
            for cell in col.cells.values():
                if cell.is_lf:
                    total += int(nx * ny * cell.ndofs[0])
        return int(total)

    def nhbr_cells_in_nhbr_col(self, col_key, cell_key, nhbr_col_key):
        """Leaf cells of column ``nhbr_col_key`` overlapping cell ``cell_key`` in
        angle: the same key, else the parent, else the two children
        (dg/mesh/nhbr_cells_in_nhbr_col.py:14-65).  Returns [k0, k1]."""
        cell = self.cols[col_key].cells[cell_key]
        cells_n = self.cols[nhbr_col_key].cells
        out = [None, None]
        same = cells_n.get(cell.key)
        if same is not None:
            if same.is_lf:
                out[0] = cell.key
            return out
        par_key = cell_key_of(int(cell.idx / 2), cell.lv - 1)
        par = cells_n.get(par_key)
        if par is not None and par.is_lf:
            out[0] = par_key
        k0 = cell_key_of(2 * cell.idx, cell.lv + 1)
        k1 = cell_key_of(2 * cell.idx + 1, cell.lv + 1)
        c0 = cells_n.get(k0)
        if c0 is None:
            return out
        if c0.is_lf:
            out[0] = k0
        c1 = cells_n.get(k1)
        if c1 is not None and c1.is_lf:
            out[1] = k1
        return out

    # -------------------------------------------------------------- refinement
    def ref_mesh(self, kind="all", form="h"):
        """Refine every column (dg/mesh/ref_mesh.py:9-17)."""
        keys = sorted(self.cols.keys())
        if kind in ("ang", "all"):
            for k in keys:
                self.ref_col(k, kind="ang", form=form)
        if kind in ("spt", "all"):
            for k in keys:
                self.ref_col(k, kind="spt", form=form)

    def ref_col(self, col_key, kind="all", form="h"):
        """Refine one column in angle (all its cells) and/or space
        (dg/mesh/ref_col.py:13-31)."""
        col = self.cols[col_key]
        assert col.is_lf
        if kind not in ("ang", "spt", "all"):
            raise ValueError("unsupported refinement kind: {}".format(kind))
        if kind in ("ang", "all"):
            for ck in sorted(col.cells.keys()):
                self.ref_cell(col_key, ck, form=form)
        if kind in ("spt", "all"):
            self.ref_col_spt(col_key, form=form)

    def ref_col_ang(self, col_key):
        col = self.cols[col_key]
        assert col.is_lf
        for ck in sorted(col.cells.keys()):
            self.ref_cell(col_key, ck)

    def ref_col_spt(self, col_key, form="h"):
        """Spatial p- and/or h-refinement of a column (dg/mesh/ref_col_spt.py:13-29)."""
        if form not in ("h", "p", "hp"):
            raise ValueError("unsupported refinement form: {}".format(form))
        if form in ("p", "hp"):
            self._ref_col_p(col_key)
        if form in ("h", "hp"):
            self._ref_col_h(col_key)

    def _ref_col_p(self, col_key):
        # dg/mesh/ref_col_spt.py:26-44: raise the degree, then fix neighbours
        # whose x-degree differs by more than one.
        col = self.cols[col_key]
        assert col.is_lf
        col.ndofs[0] += 1
        col.ndofs[1] += 1
        for face in range(4):
            for nk in list(set(col.nhbr_keys[face])):
                if nk is None:
                    continue
                nb = self.cols[nk]
                assert nb.is_lf
                if abs(col.ndofs[0] - nb.ndofs[0]) > 1:
                    self._ref_col_p(nk)

    def _ref_col_h(self, col_key):
        # dg/mesh/ref_col_spt.py:46-177: split into four children after
        # refining coarser neighbours (2:1 balance), then rewire neighbour keys.
        col = self.cols[col_key]
        assert col.is_lf
        i, j = col.idx[0], col.idx[1]
        lv = col.lv
        x0, y0, xf, yf = col.pos
        for face in range(4):
            for nk in list(set(col.nhbr_keys[face])):
                if nk is None:
                    continue
                nb = self.cols[nk]
                assert nb.is_lf
                if lv - nb.lv == 1:
                    self.ref_col(nk, kind="spt")

        kid_idx = [[2 * i, 2 * j], [2 * i + 1, 2 * j],
                   [2 * i, 2 * j + 1], [2 * i + 1, 2 * j + 1]]
        xm = (x0 + xf) / 2.
        ym = (y0 + yf) / 2.
        kid_pos = [[x0, y0, xm, ym], [x0, ym, xm, yf],
                   [xm, y0, xf, ym], [xm, ym, xf, yf]]
        kk = [col_key_of(kid_idx[c], lv + 1) for c in range(4)]
        nk = col.nhbr_keys

        def outer(face, slot, fallback):
            # A column that is its own neighbour (periodic, one column wide)
            # hands the sibling to the child instead.
            k = nk[face][slot]
            return [k, k] if k != col_key else [fallback, fallback]

        kid_nbrs = [
            [[kk[2], kk[2]], [kk[1], kk[1]], outer(2, 1, kk[2]), outer(3, 0, kk[1])],
            [[kk[3], kk[3]], outer(1, 1, kk[0]), outer(2, 0, kk[3]), [kk[0], kk[0]]],
            [outer(0, 0, kk[0]), [kk[3], kk[3]], [kk[0], kk[0]], outer(3, 1, kk[3])],
            [outer(0, 1, kk[1]), outer(1, 0, kk[2]), [kk[1], kk[1]], [kk[2], kk[2]]],
        ]
        for c in range(4):
            self.add_col(Column(kid_pos[c], kid_idx[c][:], lv + 1, True,
                                col.ndofs[:], copy.deepcopy(col.cells),
                                kid_nbrs[c][:]))

        # Neighbours now see the child that touches them.
        facing_child = [2, 3, 1, 0]
        for face in range(4):
            for slot in range(2):
                nbk = col.nhbr_keys[face][slot]
                if nbk is None:
                    continue
                nb = self.cols[nbk]
                assert nb.is_lf
                child_key = kk[facing_child[int((2 * face + slot + 1) / 2) % 4]]
                opp = (face + 2) % 4
                if nb.lv - lv == 0:
                    nb.nhbr_keys[opp][(slot + 1) % 2] = child_key
                elif nb.lv - lv == 1:
                    nb.nhbr_keys[opp][0] = child_key
                    nb.nhbr_keys[opp][1] = child_key
        self.del_col(col_key)

    def ref_cell(self, col_key, cell_key, form="h"):
        """Angular p- and/or h-refinement of one cell (dg/mesh/ref_cell.py:15-24)."""
        if form not in ("h", "p", "hp"):
            raise ValueError("unsupported refinement form: {}".format(form))
        if form in ("p", "hp"):
            self._ref_cell_p(col_key, cell_key)
        if form in ("h", "hp"):
            self._ref_cell_h(col_key, cell_key)

    def _ref_cell_p(self, col_key, cell_key):
        # dg/mesh/ref_cell.py:26-58
        col = self.cols[col_key]
        cell = col.cells[cell_key]
        assert cell.is_lf
        cell.ndofs[0] += 1
        for face in range(4):
            for nck in list(set(col.nhbr_keys[face])):
                if nck is None:
                    continue
                ncol = self.cols[nck]
                assert ncol.is_lf
                for nbk in list(set(self.nhbr_cells_in_nhbr_col(col_key, cell_key, nck))):
                    if nbk is None:
                        continue
                    nbc = ncol.cells[nbk]
                    assert nbc.is_lf
                    if abs(cell.ndofs[0] - nbc.ndofs[0]) > 1:
                        self._ref_cell_p(nck, nbk)
        for loc in ("+", "-"):
            nbc = col.nhbr_cell(cell.key, loc)
            if abs(cell.ndofs[0] - nbc.ndofs[0]) > 1:
                self._ref_cell_p(col_key, nbc.key)

    def _ref_cell_h(self, col_key, cell_key):
        # dg/mesh/ref_cell.py:60-167
        col = self.cols[col_key]
        cell = col.cells[cell_key]
        assert cell.is_lf
        idx, lv = cell.idx, cell.lv
        z0, zf = cell.pos
        quadrant = cell.quadrant

        for side in range(2):
            nbk = cell.nhbr_keys[side]
            if nbk is None:
                continue
            nbc = col.cells[nbk]
            assert nbc.is_lf
            if lv - nbc.lv == 1:
                self.ref_cell(col_key, nbk)
        for face in range(4):
            for nck in col.nhbr_keys[face]:
                if nck is None:
                    continue
                ncol = self.cols[nck]
                assert ncol.is_lf
                for nbk in self.nhbr_cells_in_nhbr_col(col_key, cell_key, nck):
                    if nbk is None:
                        continue
                    nbc = ncol.cells[nbk]
                    assert nbc.is_lf
                    if lv - nbc.lv == 1:
                        self.ref_cell(nck, nbk)

        kid_idx = [2 * idx, 2 * idx + 1]
        zm = (z0 + zf) / 2.
        kid_pos = [[z0, zm], [zm, zf]]
        if quadrant is not None:
            kid_quad = [quadrant, quadrant]
        else:
            # A child is tagged with the angular quadrant that contains it.
            quads = [[0, PI / 2], [PI / 2, PI], [PI, 3 * PI / 2], [3 * PI / 2, 2 * PI]]
            kid_quad = [None, None]
            for c, p in enumerate(kid_pos):
                for s, q in enumerate(quads):
                    if p[0] >= q[0] and p[1] <= q[1]:
                        kid_quad[c] = s
        kk = [cell_key_of(kid_idx[c], lv + 1) for c in range(2)]
        kid_nbrs = [[None, kk[1]], [kk[0], None]]
        for side in range(2):
            nbk = cell.nhbr_keys[side]
            if nbk is None:
                continue
            nbc = col.cells[nbk]
            if nbk == cell.key:
                kid_nbrs[side][side] = kid_nbrs[side][(side + 1) % 2]
            elif nbc.is_lf:
                kid_nbrs[side][side] = cell.nhbr_keys[side]
            else:
                raise RuntimeError("2-neighbour assumption violated while refining cell")
        for c in range(2):
            col.add_cell(Cell(kid_pos[c], kid_idx[c], lv + 1, True, cell.ndofs[:],
                              kid_quad[c], kid_nbrs[c][:]))
        for side, nbk in enumerate(cell.nhbr_keys):
            if nbk is not None and nbk != cell.key:
                nbc = col.cells[nbk]
                assert nbc.is_lf
                nbc.nhbr_keys[(side + 1) % 2] = kk[side]
        col.del_cell(cell_key)

    # --------------------------------------------------------------------- I/O
    def to_file(self, file_path="mesh.json"):
        """JSON layout of dg/mesh/to_file.py:10-49."""
        out = {"Ls": self.Ls, "pbcs": self.pbcs, "has_th": self.has_th, "cols": {}}
        for ck, col in self.cols.items():
            cd = {"pos": col.pos, "idx": col.idx, "lv": col.lv, "key": col.key,
                  "is_lf": col.is_lf, "ndofs": col.ndofs,
                  "nhbr_keys": col.nhbr_keys, "cells": {}}
            for kk, cell in col.cells.items():
                cd["cells"][kk] = {"pos": cell.pos, "idx": cell.idx, "lv": cell.lv,
                                   "key": cell.key, "is_lf": cell.is_lf,
                                   "ndofs": cell.ndofs, "quadrant": cell.quadrant,
                                   "nhbr_keys": cell.nhbr_keys}
            out["cols"][ck] = cd
        with open(file_path, "w") as fh:
            json.dump(out, fh)

    def __eq__(self, other):
        return (self.Ls == other.Ls and self.pbcs == other.pbcs
                and self.has_th == other.has_th and self.cols == other.cols)

    def __str__(self):
        return ("Ls     :  {}\n".format(self.Ls) +
                "pbcs   :  {}\n".format(self.pbcs) +
                "has_th :  {}\n".format(self.has_th) +
                "cols   :  {}\n".format(sorted(self.cols.keys())))


def from_dict(d):
    """Mesh from the JSON dictionary of dg/mesh/to_file.py (dg/mesh/from_file.py:13-63)."""
    mesh = Mesh(Ls=d["Ls"], pbcs=d["pbcs"], has_th=d["has_th"])
    mesh.del_col(0)
    for ck in d["cols"].keys():
        cd = d["cols"][ck]
        cells = {}
        for kk in cd["cells"].keys():
            c = cd["cells"][kk]
            cells[int(kk)] = Cell(c["pos"], c["idx"], c["lv"], c["is_lf"], c["ndofs"],
                                  c["quadrant"], c["nhbr_keys"])
        mesh.add_col(Column(cd["pos"], cd["idx"], cd["lv"], cd["is_lf"], cd["ndofs"],
                            cells, cd["nhbr_keys"]))
    return mesh


def from_file(file_path="mesh.json"):
    with open(file_path, "r") as fh:
        return from_dict(json.load(fh))


def mesh_to_dict(mesh):
    """Plain-dict snapshot in the JSON layout (keys as strings, as after a JSON
    round trip), for any mesh object with the reference's attributes."""
    d = {"Ls": list(mesh.Ls), "pbcs": list(mesh.pbcs), "has_th": mesh.has_th, "cols": {}}
    for ck, col in mesh.cols.items():
        cd = {"pos": list(col.pos), "idx": list(col.idx), "lv": col.lv, "key": col.key,
              "is_lf": col.is_lf, "ndofs": list(col.ndofs),
              "nhbr_keys": [list(x) for x in col.nhbr_keys], "cells": {}}
        for kk, cell in col.cells.items():
            cd["cells"][str(kk)] = {"pos": list(cell.pos), "idx": cell.idx, "lv": cell.lv,
                                    "key": cell.key, "is_lf": cell.is_lf,
                                    "ndofs": list(cell.ndofs), "quadrant": cell.quadrant,
                                    "nhbr_keys": list(cell.nhbr_keys)}
        d["cols"][str(ck)] = cd
    return d

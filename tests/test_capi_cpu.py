"""The C-ABI library builds, loads and exports every symbol include/rtg.h
declares; host-only entry points (quadrature, argument checks) work without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import golden_io
from rtg import _lib

HEADER = os.path.join(os.path.dirname(golden_io.GOLDEN), os.pardir, "include", "rtg.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rtg_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    lib = _lib.load()
    syms = declared_symbols()
    assert "rtg_create" in syms and "rtg_solve" in syms
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(_lib.SIGNATURES)


def test_abi_version():
    assert _lib.load().rtg_abi_version() == 1


def test_quadrature_matches_reference():
    from rtg.layout import quad
    z = np.load(golden_io.GOLDEN + "/quadrature.npz")
    for n in range(1, 13):
        x, w = quad(0, n)
        np.testing.assert_allclose(x, z["lgl_x_%d" % n], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, z["lgl_w_%d" % n], rtol=1e-14)
        x, w = quad(1, n)
        np.testing.assert_allclose(x, z["lg_x_%d" % n], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, z["lg_w_%d" % n], rtol=1e-14)


def test_quad_rejects_bad_sizes():
    lib = _lib.load()
    x = np.zeros(20)
    w = np.zeros(20)
    rc = lib.rtg_quad_nodes(0, 0, _lib.ptr(x, C.c_double), _lib.ptr(w, C.c_double))
    assert rc == _lib.RTG_ERR_SIZE
    assert b"[1, 16]" in lib.rtg_last_error()
    rc = lib.rtg_quad_nodes(2, 4, _lib.ptr(x, C.c_double), _lib.ptr(w, C.c_double))
    assert rc == _lib.RTG_ERR_ARG


def test_create_rejects_null():
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.rtg_create(None, None, 0, C.byref(h)) != 0
    assert h.value is None


def test_layout_flattening_matches_oracle_order():
    from rtg.layout import MeshLayout
    from oracle import rt_oracle as O
    mesh_fn, _ = golden_io.problem("hp_hanging")
    m = mesh_fn()
    lay = MeshLayout(m)
    L = O.Layout(m)
    assert lay.N == L.N
    for e, key in enumerate(lay.elem_keys):
        assert int(lay.elem_off[e]) == L.off[key]
    X, Y, T = lay.node_coords()
    Xo, Yo, To = O.node_coords(m)
    np.testing.assert_allclose(X, Xo, atol=1e-15)
    np.testing.assert_allclose(Y, Yo, atol=1e-15)
    np.testing.assert_allclose(T, To, atol=1e-15)

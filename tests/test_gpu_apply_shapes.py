"""Every plan shape of the apply gives the same operator: FP32 plans (items per
CTA, rows per item, split launches, scattering on the tensor cores with
TF32 hi/lo splitting) against the FP64 apply, and FP64 plans against each
other.  Meshes include columns with more than 128 angular nodes (two
tensor-core row tiles) and nx = ny = 9 (81 nodes, N padded to 96)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_SHAPES = ([(rows, gcap, split, tc) for tc in (0, 1) for rows in (16, 64) for gcap in (0, 1)
                for split in (0, 1)] + [(rows, 0, 0, 2) for rows in (16, 64)])
FP64_SHAPES = [(rows, gcap, split, 0) for rows in (16, 64) for gcap in (0, 1) for split in (0, 1)]


def _case(name):
    from rtg import workloads as W
    from rtg.mesh import Mesh
    if name == "random_hp":   # small random hp mesh, several degrees
        return (W.random_hp_mesh([3., 2.], 2, 3, rounds=3, seed=5, frac_spt=0.35, frac_ang=0.3, n_max=6,
                                 nref_ang=2, nref_spt=1), W.gaussian_bump_problem(amp=3.0))
    if name == "nth144":      # 16 angular cells of 9 nodes: 144 angular rows per column (two row tiles)
        m = Mesh([1., 1.], [False, False], [4, 4, 9], True)
        for _ in range(4):
            m.ref_mesh(kind="ang", form="h")
        m.ref_mesh(kind="spt", form="h")
        return m, W.gaussian_bump_problem(Lx=1., Ly=1., amp=2.0, xc=0.5, yc=0.5, width=0.3)
    # nx = ny = 9: 81 spatial nodes per column
    m = Mesh([1., 1.], [False, False], [9, 9, 5], True)
    for _ in range(2):
        m.ref_mesh(kind="ang", form="h")
    m.ref_mesh(kind="spt", form="h")
    return m, W.gaussian_bump_problem(Lx=1., Ly=1., amp=5.0, xc=0.3, yc=0.6, width=0.2, g=0.5)


def _shape(ctx, prec, shape):
    from rtg import _lib
    arr = None if shape is None else np.asarray(shape, dtype=np.int32)
    _lib.check(ctx.lib.rtg_apply_shape(ctx.h, prec, None if arr is None else _lib.ptr(arr, C.c_int32)))


@pytest.mark.parametrize("name", ["random_hp", "nth144", "n9"])
def test_plan_shapes_agree(name):
    import torch
    from rtg import DeviceContext, _lib
    mesh, spec = _case(name)
    ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    torch.manual_seed(0)
    x = torch.randn(ctx.N, dtype=torch.float64, device=ctx.device)
    flag_sets = {"system": _lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, "scat": _lib.RTG_SCAT}
    ref = {k: ctx.apply(f, x, prec=_lib.RTG_FP64) for k, f in flag_sets.items()}
    for shape in FP64_SHAPES:
        _shape(ctx, _lib.RTG_FP64, shape)
        for k, f in flag_sets.items():
            y = ctx.apply(f, x, prec=_lib.RTG_FP64)
            err = float(torch.linalg.norm(y - ref[k]) / torch.linalg.norm(ref[k]))
            assert err <= 1e-14, (name, shape, k, err)
    xf = x.float()
    for shape in FP32_SHAPES:
        _shape(ctx, _lib.RTG_FP32, shape)
        for k, f in flag_sets.items():
            y = ctx.apply(f, xf, prec=_lib.RTG_FP32).double()
            err = float(torch.linalg.norm(y - ref[k]) / torch.linalg.norm(ref[k]))
            # FP32 arithmetic; the tensor-core product splits each operand into
            # TF32 hi + lo parts (about 2^-21 relative per product)
            assert err < 2e-6, (name, shape, k, err)
    # back to the autotuned plans
    _shape(ctx, _lib.RTG_FP32, None)
    _shape(ctx, _lib.RTG_FP64, None)
    y = ctx.apply(flag_sets["system"], xf, prec=_lib.RTG_FP32).double()
    assert float(torch.linalg.norm(y - ref["system"]) / torch.linalg.norm(ref["system"])) < 2e-6


def test_bad_shape_rejected():
    from rtg import DeviceContext, _lib, workloads as W
    mesh = W.config1_mesh()
    spec = W.manufactured_problem()
    ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    for prec, shape in ((_lib.RTG_FP64, (16, 0, 0, 1)), (_lib.RTG_FP32, (0, 0, 0, 0)),
                        (_lib.RTG_FP32, (16, -1, 0, 0)), (_lib.RTG_FP32, (16, 0, 2, 0)),
                        (_lib.RTG_FP32, (16, 0, 0, 3)), (_lib.RTG_FP64, (16, 0, 0, 2))):
        arr = np.asarray(shape, dtype=np.int32)
        assert ctx.lib.rtg_apply_shape(ctx.h, prec, _lib.ptr(arr, C.c_int32)) == _lib.RTG_ERR_ARG

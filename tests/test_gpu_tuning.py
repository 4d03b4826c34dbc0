"""The FP32 apply autotuner: every degree class of columns is timed with each
candidate item size and the fastest is kept; the tuned apply still matches the
FP64 apply."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CANDIDATES = (16, 32, 64, 128)


def test_tuning_table_and_tuned_apply():
    import torch
    from rtg import DeviceContext, _lib, workloads as W
    mesh = W.random_hp_mesh([3., 2.], 2, 3, rounds=3, seed=5, frac_spt=0.35, frac_ang=0.3, n_max=6,
                            nref_ang=2, nref_spt=1)
    spec = W.gaussian_bump_problem(amp=3.0)
    ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    table = np.zeros((256, 8), dtype=np.int32)
    ncls = C.c_int()
    _lib.check(ctx.lib.rtg_apply_tuning(ctx.h, _lib.ptr(table, C.c_int32), 256, C.byref(ncls), None))
    n = ncls.value
    assert n >= 2
    nx_ny_classes = {(c.ndofs[0], c.ndofs[1]) for c in mesh.cols.values()}
    assert {(int(r[0]), int(r[1])) for r in table[:n]} == nx_ny_classes
    for r in table[:n]:
        cap = abs(int(r[3]))       # negative: the default plan won overall
        assert cap in CANDIDATES
        times = [t for t in r[4:] if t >= 0]
        assert times and r[4 + CANDIDATES.index(cap)] <= min(times) / 0.97 + 1
    x = torch.randn(ctx.N, dtype=torch.float64, device=ctx.device)
    fl = _lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS
    y64 = ctx.apply(fl, x, prec=_lib.RTG_FP64)
    y32 = ctx.apply(fl, x.float(), prec=_lib.RTG_FP32)
    assert float(torch.linalg.norm(y32.double() - y64) / torch.linalg.norm(y64)) < 2e-6

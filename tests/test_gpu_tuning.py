"""The apply autotuner: every plan shape of the candidate list (rows per work
item, one CTA per column or per item, one launch or one per shared-memory
class, scattering on CUDA cores or tensor cores) is timed and the fastest is
kept; the tuned FP32 apply matches the FP64 apply."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROWS = (16, 32, 64)


def test_tuning_table_and_tuned_apply():
    import torch
    from rtg import DeviceContext, _lib, workloads as W
    mesh = W.random_hp_mesh([3., 2.], 2, 3, rounds=3, seed=5, frac_spt=0.35, frac_ang=0.3, n_max=6,
                            nref_ang=2, nref_spt=1)
    spec = W.gaussian_bump_problem(amp=3.0)
    ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    table = np.zeros((256, 9), dtype=np.int32)
    n = C.c_int()
    _lib.check(ctx.lib.rtg_apply_tuning(ctx.h, _lib.ptr(table, C.c_int32), 256, C.byref(n), None))
    rec = table[:n.value]
    assert len(rec) == 14
    assert {tuple(int(v) for v in r[:4]) for r in rec} == ({(q, g, s, 0) for q in ROWS for g in (0, 1)
                                                            for s in (0, 1)} |
                                                           {(32, 0, 0, 2), (64, 0, 0, 2)})
    assert int(rec[:, 4].sum()) == 1
    chosen = rec[rec[:, 4] == 1][0]
    assert chosen[5] == rec[:, 5].min()
    for r in rec:
        assert r[5] > 0 and r[6] > 0 and r[7] > 0 and r[8] >= 1
        if r[1] == 1:
            assert r[7] == r[6]                       # one CTA per item
        else:
            assert r[7] <= min(len(mesh.cols), r[6])   # at most one CTA per column
        if r[3] >= 1:
            assert r[8] >= 2                          # the tensor-core launch beside the tiled ones
    x = torch.randn(ctx.N, dtype=torch.float64, device=ctx.device)
    fl = _lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS
    y64 = ctx.apply(fl, x, prec=_lib.RTG_FP64)
    y32 = ctx.apply(fl, x.float(), prec=_lib.RTG_FP32)
    assert float(torch.linalg.norm(y32.double() - y64) / torch.linalg.norm(y64)) < 2e-6

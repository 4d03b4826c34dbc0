"""rtg_dots_noalloc: allocation-free inner products.

Callers that may not allocate device memory (a host whose memory manager owns
every device allocation, or a caller running its own Krylov loop around
rtg_apply where cudaMalloc would stall or break the surrounding work) get the
solver's kind of inner-product reduction with its scratch in a static device
array.
This test checks it against the norms the existing entry point rtg_solve
reports for the same vectors (||b|| and the final true residual ||b - A x||),
on two calls in a row.  The file is collected last so that a run stopping at
the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_noalloc_dots_match_solver_norms():
    import torch
    from rtg import Problem, _lib

    mesh_fn, prob_fn = golden_io.problem("cfg1")
    spec = prob_fn()
    mesh = mesh_fn()
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    ctx = prob.context(mesh)
    lib = ctx.lib
    N = ctx.N
    f = ctx.forcing(spec.f)
    g = ctx.inflow(spec.bcs_dirac)
    u, info = ctx.solve(f, g, method=0, rtol=1e-10, precond=1)

    def p(t):
        return C.c_void_p(t.data_ptr())

    # b = mask_I (f - A mask_B g), r = b - mask_I A mask_I u  (existing entry points)
    gb = torch.empty_like(g)
    t = torch.empty_like(g)
    b = torch.empty_like(f)
    ui = torch.empty_like(u)
    _lib.check(lib.rtg_mask_vector(ctx.h, 1, p(g), p(gb), None))
    _lib.check(lib.rtg_apply(ctx.h, _lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, _lib.RTG_FP64, p(gb), p(t), None))
    _lib.check(lib.rtg_mask_vector(ctx.h, 0, p(f), p(b), None))
    b -= t
    _lib.check(lib.rtg_mask_vector(ctx.h, 0, p(u), p(ui), None))
    _lib.check(lib.rtg_apply(ctx.h, _lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, _lib.RTG_FP64, p(ui), p(t), None))
    r = b - t
    torch.cuda.synchronize()

    out = torch.full((2,), float("nan"), dtype=torch.float64, device=ctx.device)
    for call in range(2):
        out.fill_(float("nan"))
        _lib.check(lib.rtg_dots_noalloc(1, p(b), 0, p(b), N, p(out), None))
        _lib.check(lib.rtg_dots_noalloc(1, p(r), 0, p(r), N, p(out[1:]), None))
        torch.cuda.synchronize()
        bb, rr = out.cpu().numpy()
        assert abs(np.sqrt(bb) - info["rhs_norm"]) <= TOL * info["rhs_norm"], (call, np.sqrt(bb), info["rhs_norm"])
        assert abs(np.sqrt(rr) - info["res_f"]) <= TOL * info["rhs_norm"], (call, np.sqrt(rr), info["res_f"])

    # several vectors at once: V = [b; r] against w = b
    V = torch.stack([b, r]).contiguous()
    for call in range(2):
        out.fill_(float("nan"))
        _lib.check(lib.rtg_dots_noalloc(2, p(V), N, p(b), N, p(out), None))
        torch.cuda.synchronize()
        ref = (V @ b).cpu().numpy()
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=TOL, atol=TOL * float(b @ b))


def test_noalloc_rejects_sizes_beyond_maximum():
    import torch
    from rtg import _lib
    lib = _lib.load()
    x = torch.ones(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(65, dtype=torch.float64, device="cuda")
    rc = lib.rtg_dots_noalloc(65, C.c_void_p(x.data_ptr()), 0, C.c_void_p(x.data_ptr()), 16,
                              C.c_void_p(out.data_ptr()), None)
    assert rc == _lib.RTG_ERR_SIZE
    assert b"[1, 64]" in lib.rtg_last_error()


@pytest.mark.parametrize("k,pad", [(9, 0), (17, 5), (64, 3)])
def test_noalloc_many_vectors(k, pad):
    """Vector counts that exercise a last group of fewer than eight, several
    groups, and the whole 64-wide scratch row, with rows ldv = n + pad apart;
    two calls in a row against torch's V @ w."""
    import torch
    from rtg import _lib
    lib = _lib.load()
    n = 100003
    gen = torch.Generator(device="cuda").manual_seed(k)
    Vp = torch.randn(k, n + pad, dtype=torch.float64, device="cuda", generator=gen)
    w = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
    ref = (Vp[:, :n] @ w).cpu().numpy()
    out = torch.empty(k, dtype=torch.float64, device="cuda")
    for call in range(2):
        out.fill_(float("nan"))
        _lib.check(lib.rtg_dots_noalloc(k, C.c_void_p(Vp.data_ptr()), n + pad, C.c_void_p(w.data_ptr()), n,
                                        C.c_void_p(out.data_ptr()), None))
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * np.sqrt(n) * 4)

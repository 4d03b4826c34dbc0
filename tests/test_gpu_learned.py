"""GPU parity of the learned sweep correction against its CPU oracle: features,
forward pass, training targets, expansion, loss and gradient, and the Adam
step; then training and the flexible solve that uses the network.

Tolerances: the kernels run in FP32 (the oracle in float64 with the same
BF16-rounded weights), so values match to ~1e-5 relative and gradients to
1e-4 relative (2-norm)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    from rtg import DeviceContext, workloads as W
    from oracle import nn_oracle as NO
    mesh = W.small_random_mesh()
    spec = W.gaussian_bump_problem(amp=5.0, width=0.3, g=0.7)
    ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    rl = NO.RowLayout(mesh, spec.kappa, spec.sigma)
    assert rl.N == ctx.N
    return torch, ctx, rl, spec


def _params(seed):
    from rtg import learned as LN
    rng = np.random.default_rng(seed)
    p = LN.init_params(seed)
    p += (rng.standard_normal(p.size) * 0.05).astype(np.float32)
    return p


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_row_count(setup):
    from rtg import learned as LN
    torch, ctx, rl, _ = setup
    assert LN.rows(ctx) == len(rl.rows)


def test_physics_features_match_oracle(setup):
    from rtg import learned as LN
    torch, ctx, rl, _ = setup
    F = LN.features(ctx).cpu().numpy().astype(np.float64)
    Fo = rl.physics()
    err = np.abs(F - Fo).max(axis=0) / np.maximum(np.abs(Fo).max(axis=0), 1.0)
    assert err.max() < 2e-5, err


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_moments_match_oracle(setup, prec):
    from rtg import learned as LN
    torch, ctx, rl, _ = setup
    rng = np.random.default_rng(2)
    z = rng.standard_normal(rl.N) * (1.0 + 3.0 * rng.random(rl.N))
    dt = torch.float64 if prec == "fp64" else torch.float32
    zt = torch.as_tensor(z, dtype=dt, device=ctx.device)
    M, s = LN.moments(ctx, zt)
    Mo, so = rl.moments(zt.double().cpu().numpy())
    assert abs(float(s[0]) - so) <= 1e-6 * so
    Mg = M.cpu().numpy().astype(np.float64)
    err = np.abs(Mg - Mo / so).max(axis=0) / np.maximum(np.abs(Mo / so).max(axis=0), 1.0)
    assert err.max() < 2e-5, err


def test_targets_and_correction_match_oracle(setup):
    from rtg import learned as LN
    torch, ctx, rl, _ = setup
    rng = np.random.default_rng(3)
    z = rng.standard_normal(rl.N) * rl.mask
    e = z + 0.3 * rng.standard_normal(rl.N) * rl.mask
    zt = torch.as_tensor(z, device=ctx.device)
    et = torch.as_tensor(e, device=ctx.device)
    _, s = LN.moments(ctx, zt)
    S = LN.targets(ctx, zt, et, s, 0.25).cpu().numpy().astype(np.float64)
    So = rl.stats(z, e, float(s[0]), 0.25)
    assert np.abs(S[:, :10] - So).max() <= 1e-5 * np.abs(So).max()
    assert np.all(S[:, 10:] == 0.)
    coef = rng.standard_normal((len(rl.rows), 24)).astype(np.float32)
    for dt in (torch.float64, torch.float32):
        zz = zt.to(dt).clone()
        LN.correct(ctx, torch.as_tensor(coef, device=ctx.device), zz)
        d = (zz.double() - zt.to(dt).double()).cpu().numpy()
        do = rl.correction(coef.astype(np.float64), zt.to(dt).double().cpu().numpy())
        assert _rel(d, do) < 1e-5, dt


def test_forward_matches_oracle(setup):
    from rtg import learned as LN
    from oracle import nn_oracle as NO
    torch, ctx, rl, _ = setup
    rng = np.random.default_rng(4)
    F = torch.as_tensor(rng.standard_normal((len(rl.rows), 16)).astype(np.float32), device=ctx.device)
    p = _params(5)
    O = LN.forward(torch.as_tensor(p, device=ctx.device), F).cpu().numpy()
    Oo, _ = NO.forward(NO.device_params(p), F.cpu().numpy().astype(np.float64))
    assert np.abs(O - Oo).max() <= 1e-5 * max(1.0, np.abs(Oo).max())


def test_loss_grad_matches_oracle(setup):
    """The hand-written backward pass against the oracle's gradient."""
    from rtg import learned as LN
    from oracle import nn_oracle as NO
    torch, ctx, rl, _ = setup
    rng = np.random.default_rng(6)
    z = rng.standard_normal(rl.N) * rl.mask
    e = z + rng.standard_normal(rl.N) * rl.mask
    zt = torch.as_tensor(z, device=ctx.device)
    F = LN.features(ctx)
    M, s = LN.moments(ctx, zt)
    S = LN.targets(ctx, zt, torch.as_tensor(e, device=ctx.device), s, 1.0 / rl.N)
    p = _params(7)
    tr = LN.Trainer(ctx.device)
    loss, grad = tr.loss_grad(torch.as_tensor(p, device=ctx.device), F, M, S)
    lo, go = NO.loss_grad(NO.device_params(p), F.cpu().numpy().astype(np.float64),
                          M.cpu().numpy().astype(np.float64), S.cpu().numpy().astype(np.float64)[:, :10])
    assert abs(float(loss[0]) - lo) <= 1e-5 * abs(lo)
    g = grad.cpu().numpy().astype(np.float64)
    assert _rel(g, go) < 1e-4
    # every parameter block individually
    off = 0
    for name, shp in NO.SHAPES:
        n = int(np.prod(shp))
        if np.linalg.norm(go[off:off + n]) > 1e-8 * np.linalg.norm(go):
            assert _rel(g[off:off + n], go[off:off + n]) < 1e-3, name
        off += n


def test_adam_matches_oracle(setup):
    from rtg import learned as LN
    from oracle import nn_oracle as NO
    torch, ctx, rl, _ = setup
    rng = np.random.default_rng(8)
    p = rng.standard_normal(NO.NPARAM).astype(np.float32)
    g = rng.standard_normal(NO.NPARAM).astype(np.float32)
    m = (rng.standard_normal(NO.NPARAM) * 0.1).astype(np.float32)
    v = (rng.random(NO.NPARAM) * 0.1).astype(np.float32)
    P, Mt, Vt = (torch.as_tensor(a, device=ctx.device).clone() for a in (p, m, v))
    tr = LN.Trainer(ctx.device)
    tr.grad.copy_(torch.as_tensor(g, device=ctx.device))
    tr.adam(P, Mt, Vt, 3, 1e-2, wd=1e-4)
    po, mo, vo = NO.adam(p.astype(np.float64), g.astype(np.float64), m.astype(np.float64), v.astype(np.float64),
                         3, 1e-2, wd=1e-4)
    assert np.abs(P.cpu().numpy() - po).max() < 1e-5
    assert np.abs(Mt.cpu().numpy() - mo).max() < 1e-6
    assert np.abs(Vt.cpu().numpy() - vo).max() < 1e-6


@pytest.fixture(scope="module")
def trained(setup):
    from rtg import learned as LN
    torch, ctx, rl, spec = setup
    f = ctx.forcing(spec.f)
    g = ctx.inflow(spec.bcs_dirac)
    F, M, S = LN.stack(LN.collect_pairs(ctx, f, g, n_pairs=8))
    P1, h1 = LN.train(F, M, S, steps=300, batch=8192, lr=2e-3, seed=0, log_every=50)
    P2, _ = LN.train(F, M, S, steps=300, batch=8192, lr=2e-3, seed=0)
    return F, M, S, P1, P2, h1, f, g


def test_training_reduces_loss_and_is_deterministic(setup, trained):
    from rtg import learned as LN
    torch, ctx, rl, _ = setup
    F, M, S, P1, P2, hist, _, _ = trained
    before = LN.evaluate(torch.as_tensor(LN.init_params(0), device=ctx.device), F, M, S)
    after = LN.evaluate(P1, F, M, S)
    assert 0.9 < before < 1.1          # near-zero coefficients leave the sweep's error
    assert after < 0.8 * before, (before, after, hist)
    assert torch.equal(P1, P2)         # fixed seed, fixed-order reductions


@pytest.mark.parametrize("method", [0, 1])
def test_learned_flexible_solve_matches_plain(setup, trained, method):
    """FGMRES with the learned correction converges to the FP64 solution."""
    from rtg import learned as LN
    torch, ctx, rl, _ = setup
    _, _, _, P1, _, _, f, g = trained
    LN.set_params(ctx, P1)
    u0, i0 = ctx.solve(f, g, method=0, precond=1, rtol=1e-13, restart=30)
    u1, i1 = ctx.solve(f, g, method=method, precond=3, rtol=1e-12, restart=30, inner_rtol=1e-5)
    assert i0["converged"] and i1["converged"]
    assert i1["learned"] > 0
    err = float(torch.linalg.norm(u1 - u0) / torch.linalg.norm(u0))
    assert err < 1e-10, (err, i1)


def test_learned_precondition_entry_point(setup, trained):
    """rtg_nn_precondition = sweep, then correct() with the network's coefficients."""
    import ctypes as C
    from rtg import learned as LN, _lib
    torch, ctx, rl, _ = setup
    _, _, _, P1, _, _, _, _ = trained
    LN.set_params(ctx, P1)
    rng = np.random.default_rng(9)
    r = torch.as_tensor(rng.standard_normal(rl.N) * rl.mask, dtype=torch.float32, device=ctx.device)
    z = torch.empty_like(r)
    _lib.check(ctx.lib.rtg_nn_precondition(ctx.h, _lib.RTG_FP32, C.c_void_p(r.data_ptr()),
                                           C.c_void_p(z.data_ptr()), None))
    z0 = ctx.precondition(r, prec=_lib.RTG_FP32)
    coef = LN.forward(P1, LN.features(ctx))
    LN.correct(ctx, coef, z0)
    torch.cuda.synchronize()
    assert float((z - z0).abs().max()) <= 1e-6 * float(z0.abs().max())
    mask = torch.as_tensor(rl.mask, device=ctx.device)
    assert float(z[~mask].abs().max()) == 0.0
    # linear in r
    z2 = torch.empty_like(r)
    r2 = (-2.5 * r).contiguous()
    _lib.check(ctx.lib.rtg_nn_precondition(ctx.h, _lib.RTG_FP32, C.c_void_p(r2.data_ptr()),
                                           C.c_void_p(z2.data_ptr()), None))
    torch.cuda.synchronize()
    assert float((z2 + 2.5 * z).abs().max()) <= 1e-5 * float(z2.abs().max())


def test_precond3_without_network_is_an_error(setup):
    from rtg import DeviceContext, _lib, workloads as W
    torch, ctx, rl, spec = setup
    mesh = W.small_random_mesh(seed=4)
    c2 = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
    f = c2.forcing(spec.f)
    g = c2.inflow(spec.bcs_dirac)
    with pytest.raises(_lib.RtgError) as ei:
        c2.solve(f, g, method=1, precond=3)
    assert ei.value.code == _lib.RTG_ERR_ARG

"""The CPU oracle of the learned correction, pinned on its own: its analytic
gradient matches central finite differences of its loss (float64), its BF16
rounding is round-to-nearest-even, the correction is linear in z, and the
per-row statistics reproduce the squared error of the correction."""
import numpy as np

from oracle import nn_oracle as NO


def _small_case():
    from rtg import workloads as W
    mesh = W.small_random_mesh()
    spec = W.gaussian_bump_problem(amp=5.0, width=0.3, g=0.7)
    return mesh, spec


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3, 0.0], dtype=np.float32)
    r = NO.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa is 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == -2.5 and r[5] == 0.0
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def _random_stats(rng, R):
    S = np.zeros((R, 10))
    for r in range(R):
        B = rng.standard_normal((3, 5))
        t = rng.standard_normal(5)
        G = B @ B.T
        q = B @ t
        S[r] = [G[0, 0], G[0, 1], G[0, 2], G[1, 1], G[1, 2], G[2, 2], q[0], q[1], q[2], t @ t]
    return S


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    R = 24
    F = rng.standard_normal((R, NO.N_IN))
    M = rng.standard_normal((R, NO.N_MOM))
    S = _random_stats(rng, R)
    p = np.concatenate([rng.standard_normal(n) * sc for n, sc in
                        [(NO.N_IN * NO.N_HID, 0.3), (NO.N_HID, 0.1), (NO.N_HID * NO.N_HID, 0.1),
                         (NO.N_HID, 0.1), (NO.N_HID * NO.N_OUT, 0.1), (NO.N_OUT, 0.1)]])
    loss, g = NO.loss_grad(p, F, M, S)
    idx = rng.choice(NO.NPARAM, 60, replace=False)
    h = 1e-6
    for i in idx:
        d = np.zeros_like(p)
        d[i] = h
        fd = (NO.loss_grad(p + d, F, M, S)[0] - NO.loss_grad(p - d, F, M, S)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-7 * abs(loss), (i, fd, g[i])


def test_correction_linear_and_stats_consistent():
    mesh, spec = _small_case()
    rl = NO.RowLayout(mesh, spec.kappa, spec.sigma)
    rng = np.random.default_rng(1)
    z1 = rng.standard_normal(rl.N) * rl.mask
    z2 = rng.standard_normal(rl.N) * rl.mask
    coef = rng.standard_normal((len(rl.rows), NO.N_OUT))
    d = rl.correction(coef, 2.0 * z1 - 3.0 * z2)
    assert np.abs(d - (2.0 * rl.correction(coef, z1) - 3.0 * rl.correction(coef, z2))).max() < 1e-11 * np.abs(d).max()
    assert np.all(d[~rl.mask] == 0.)
    F = rl.physics()
    assert F.shape == (len(rl.rows), NO.N_IN) and np.all(np.isfinite(F))
    # sum_rows o^T G o - 2 q^T o + c with o = C m/s equals |L z - (e - z)|^2 / s^2
    e = z1 + rng.standard_normal(rl.N) * rl.mask
    M, s = rl.moments(z1)
    S = rl.stats(z1, e, s, 1.0)
    direct = float(np.sum((rl.correction(coef, z1) - (e - z1)) ** 2)) / s ** 2
    o = np.einsum("rkl,rl->rk", coef.reshape(-1, 3, NO.N_MOM), M / s)
    G = np.zeros((len(S), 3, 3))
    for k, a, b in [(0, 0, 0), (1, 0, 1), (2, 0, 2), (3, 1, 1), (4, 1, 2), (5, 2, 2)]:
        G[:, a, b] = S[:, k]
        G[:, b, a] = S[:, k]
    quad = float(np.einsum("ra,rab,rb->", o, G, o) - 2 * (S[:, 6:9] * o).sum() + S[:, 9].sum())
    assert abs(quad - direct) <= 1e-9 * max(1.0, direct)

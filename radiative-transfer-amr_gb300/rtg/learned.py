"""Learned correction of the sweep preconditioner: data, training, storage.

The correction and its kernels live in librtg (csrc/rtg_nn.cu, declared in
include/rtg.h); this module drives them.  Torch tensors only carry device
buffers: every feature, moment, forward, loss, gradient and Adam update runs
in the library's own CUDA kernels.

Preconditioner 3 is M r = z + L z, z = P_sweep^{-1} r, with L linear in z: per
row (element, spatial node) o = C m(z), C a 3 x 8 coefficient matrix that a
network computes from 16 local physics features, m(z) eight angular and
neighbour moments of z, and (L z) = o0 + o1 cos th + o2 sin th.

Data are residual -> error pairs that the method's own GMRES produces
(collect_pairs): the Arnoldi vectors v of sweep-preconditioned GMRES with
their errors e = A_II^{-1} v, or the residuals of GMRES iterates with their
errors.  Each pair becomes rows of (physics features, moments m(z)/s of the
FP32 sweep output z, statistics of the target (e - z)/s).  The loss of a pair
is sum_beta ((L z)_beta - (e - z)_beta)^2 / s^2, normalised by default so that
each pair's loss with L = 0 (the sweep alone, "loss0") is 1/npairs."""

import ctypes as C
import json
import math
import os

import numpy as np

from . import _lib
from .problem import _stream_ptr, _torch

NPARAM = _lib.RTG_NN_NPARAM
N_IN, N_HID, N_MOM, N_OUT, N_ST = (_lib.RTG_NN_IN, _lib.RTG_NN_HIDDEN, _lib.RTG_NN_MOM, _lib.RTG_NN_OUT,
                                   _lib.RTG_NN_STATS)
SYSTEM_MASKED = _lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS


def _p(t):
    return C.c_void_p(t.data_ptr())


def init_params(seed=0):
    """He-initialised hidden layers and a small output layer: the coefficients
    start near zero, i.e. M starts near the sweep alone."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((N_IN, N_HID)) * math.sqrt(2. / N_IN)
    W2 = rng.standard_normal((N_HID, N_HID)) * math.sqrt(2. / N_HID)
    W3 = rng.standard_normal((N_HID, N_OUT)) * 1e-3
    parts = [W1, np.zeros(N_HID), W2, np.zeros(N_HID), W3, np.zeros(N_OUT)]
    p = np.concatenate([a.reshape(-1) for a in parts]).astype(np.float32)
    assert p.size == NPARAM
    return p


def rows(ctx):
    n = C.c_int64()
    _lib.check(ctx.lib.rtg_nn_rows(ctx.h, C.byref(n)))
    return int(n.value)


def set_params(ctx, params):
    torch = _torch()
    p = torch.as_tensor(np.asarray(params, dtype=np.float32) if not isinstance(params, torch.Tensor)
                        else params, dtype=torch.float32).to(ctx.device).contiguous()
    _lib.check(ctx.lib.rtg_nn_set_params(ctx.h, _p(p), _stream_ptr()))
    torch.cuda.synchronize(ctx.device)


def _prec(t):
    torch = _torch()
    return _lib.RTG_FP64 if t.dtype == torch.float64 else _lib.RTG_FP32


def features(ctx):
    """Physics features of the handle's rows [rows][16]."""
    torch = _torch()
    F = torch.empty((rows(ctx), N_IN), dtype=torch.float32, device=ctx.device)
    _lib.check(ctx.lib.rtg_nn_features(ctx.h, _p(F), _stream_ptr()))
    return F


def moments(ctx, z):
    """m(z)/s per row [rows][8] and s = rms(z)."""
    torch = _torch()
    M = torch.empty((rows(ctx), N_MOM), dtype=torch.float32, device=ctx.device)
    s = torch.empty(1, dtype=torch.float32, device=ctx.device)
    _lib.check(ctx.lib.rtg_nn_moments(ctx.h, _prec(z), _p(z), _p(M), _p(s), _stream_ptr()))
    return M, s


def forward(params, F):
    """Coefficients [rows][24] of the rows with physics features F."""
    torch = _torch()
    O = torch.empty((F.shape[0], N_OUT), dtype=torch.float32, device=F.device)
    _lib.check(_lib.load().rtg_nn_forward(_p(params), _p(F), F.shape[0], _p(O), _stream_ptr()))
    return O


def correct(ctx, coef, z):
    """z += L z with the given coefficients (in place)."""
    _lib.check(ctx.lib.rtg_nn_correct(ctx.h, _prec(z), _p(coef), _p(z), _stream_ptr()))
    return z


def targets(ctx, z, e, s, weight):
    torch = _torch()
    S = torch.empty((rows(ctx), N_ST), dtype=torch.float32, device=ctx.device)
    _lib.check(ctx.lib.rtg_nn_targets(ctx.h, _prec(z), _p(z), _p(e), _p(s), C.c_float(weight), _p(S),
                                      _stream_ptr()))
    return S


class Trainer:
    """Loss, gradient and Adam through the library's kernels."""

    def __init__(self, device):
        torch = _torch()
        self.lib = _lib.load()
        self.device = device
        self.work = torch.empty(int(self.lib.rtg_nn_work_floats()), dtype=torch.float32, device=device)
        self.grad = torch.zeros(NPARAM, dtype=torch.float32, device=device)
        self.loss = torch.zeros(1, dtype=torch.float64, device=device)

    def loss_grad(self, params, F, M, S):
        _lib.check(self.lib.rtg_nn_loss_grad(_p(params), _p(F), _p(M), _p(S), F.shape[0], _p(self.work),
                                             _p(self.grad), _p(self.loss), _stream_ptr()))
        return self.loss, self.grad

    def adam(self, params, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.):
        _lib.check(self.lib.rtg_nn_adam(_p(params), _p(self.grad), _p(m), _p(v), step, C.c_float(lr),
                                        C.c_float(b1), C.c_float(b2), C.c_float(eps), C.c_float(wd),
                                        _stream_ptr()))


def _pair_rows(ctx, F, r, e, npairs, normalize):
    """Rows of one residual -> error pair: (F, m(z)/s, statistics of (e - z)/s)
    with z = P_sweep^{-1} r in FP32, weighted so that the pair's loss with
    L = 0 is 1/npairs (normalize) or sum (e - z)^2 / (s^2 npairs)."""
    z = ctx.precondition(r.float(), prec=_lib.RTG_FP32)
    M, s = moments(ctx, z)
    S = targets(ctx, z, e.float(), s, 1.0)
    l0 = float(S[:, 9].double().sum())
    if not l0 > 0.:
        return None
    S.mul_(1.0 / (npairs * (l0 if normalize else 1.0)))
    return F, M, S


def system_rhs(ctx, f_dev, g_dev):
    """b = mask_I (f - A mask_B g), the right-hand side rtg_solve solves for."""
    torch = _torch()
    mask = ctx.interior_mask()
    gB = torch.where(mask, torch.zeros_like(g_dev), g_dev)
    t = ctx.apply(SYSTEM_MASKED, gB)
    return torch.where(mask, f_dev - t, torch.zeros_like(f_dev))


def collect_pairs(ctx, f_dev, g_dev, n_pairs=12, cycle=2, rtol=1e-12, restart=30, kind="arnoldi",
                  normalize=True, max_it=1500):
    """Residual -> error pairs that the method's own sweep-GMRES generates.

    kind "arnoldi": the Arnoldi vectors v_j of sweep-preconditioned GMRES on
    the problem (the vectors a flexible method applies its preconditioner
    to), with e_j = A_II^{-1} v_j from a converged sweep-GMRES solve each.
    kind "iterates": the residuals r_j = A_II e_j of the iterates u_j of short
    GMRES cycles, e_j = u* - u_j.
    Vectors whose error solve does not converge within max_it iterations are
    skipped.  Returns a list of (F, M, S) row tensors, one entry per pair."""
    torch = _torch()
    mask = ctx.interior_mask()
    pairs = []
    if kind == "arnoldi":
        b = system_rhs(ctx, f_dev, g_dev)
        V = [b / torch.linalg.norm(b)]
        for _ in range(n_pairs - 1):
            w = ctx.apply(SYSTEM_MASKED, ctx.precondition(V[-1]))
            for _ in range(2):
                for v in V:
                    w = w - torch.dot(v, w) * v
            nw = torch.linalg.norm(w)
            if not float(nw) > 0.:
                break
            V.append(w / nw)
        zero = torch.zeros_like(g_dev)
        for v in V:
            e, inf = ctx.solve(v, zero, method=0, precond=1, rtol=rtol, restart=restart, max_it=max_it)
            if not inf["converged"]:
                continue   # no exact error for this vector (stagnating solve): no pair
            pairs.append((v, torch.where(mask, e, torch.zeros_like(e))))
    elif kind == "iterates":
        u_star, inf = ctx.solve(f_dev, g_dev, method=0, precond=1, rtol=rtol, restart=restart, max_it=max_it)
        if not inf["converged"]:
            return []   # no converged solution to measure errors against
        u = None
        for _ in range(n_pairs):
            u, _ = ctx.solve(f_dev, g_dev, method=0, precond=1, rtol=1e-300, restart=cycle, max_it=cycle, x0=u)
            e = torch.where(mask, u_star - u, torch.zeros_like(u))
            if not float(e.abs().max()) > 0.:
                break
            pairs.append((ctx.apply(SYSTEM_MASKED, e), e))
    else:
        raise ValueError("unknown pair kind {}".format(kind))
    F = features(ctx)
    out = []
    for r, e in pairs:
        rows_ = _pair_rows(ctx, F, r, e, len(pairs), normalize)
        if rows_ is not None:
            out.append(rows_)
    return out


def stack(data):
    """Concatenate (F, M, S) lists from collect_pairs into row tensors."""
    torch = _torch()
    return (torch.cat([d[0] for d in data]).contiguous(), torch.cat([d[1] for d in data]).contiguous(),
            torch.cat([d[2] for d in data]).contiguous())


def loss0(S):
    """The loss with a zero correction (the sweep alone)."""
    return float(S[:, 9].double().sum())


def train(F, M, S, steps=2000, batch=32768, lr=2e-3, seed=0, params=None, log_every=0, wd=0., log=None):
    """Adam over random row batches; lr decays by cosine to lr/20.
    Returns (params tensor, history of (step, batch loss / batch loss0))."""
    torch = _torch()
    dev = F.device
    p0 = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
    P = torch.as_tensor(p0).to(dev).contiguous()
    m = torch.zeros_like(P)
    v = torch.zeros_like(P)
    tr = Trainer(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    nrows = F.shape[0]
    hist = []
    for step in range(1, steps + 1):
        if batch >= nrows:
            Fb, Mb, Sb = F, M, S
        else:
            idx = torch.randint(0, nrows, (batch,), device=dev, generator=gen)
            Fb = F.index_select(0, idx).contiguous()
            Mb = M.index_select(0, idx).contiguous()
            Sb = S.index_select(0, idx).contiguous()
        tr.loss_grad(P, Fb, Mb, Sb)
        lr_t = lr * (0.05 + 0.95 * 0.5 * (1. + math.cos(math.pi * (step - 1) / max(1, steps))))
        tr.adam(P, m, v, step, lr_t, wd=wd)
        if log_every and (step % log_every == 0 or step == 1 or step == steps):
            l0 = float(Sb[:, 9].double().sum())
            rel = float(tr.loss[0]) / l0 if l0 > 0 else float("nan")
            hist.append((step, rel))
            if log:
                log("step {:5d}  loss/loss0 {:.4f}".format(step, rel))
    return P, hist


def evaluate(params, F, M, S):
    """Loss / loss0 over all rows for the given parameters."""
    tr = Trainer(F.device)
    tr.loss_grad(params, F, M, S)
    l0 = loss0(S)
    return float(tr.loss[0]) / l0 if l0 > 0 else float("nan")


def save(path, params, meta=None):
    p = params.detach().cpu().numpy() if hasattr(params, "detach") else np.asarray(params)
    np.savez(path, params=p.astype(np.float32), meta=json.dumps(meta or {}))


def load(path):
    d = np.load(path, allow_pickle=False)
    return d["params"].astype(np.float32), json.loads(str(d["meta"]))


DEFAULT_NET = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nets", "sweep_correction.npz")

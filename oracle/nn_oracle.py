"""CPU oracle of the learned sweep correction -- TEST INFRASTRUCTURE ONLY.

The reference has no learned preconditioner; this file restates, in float64
numpy, the math that librtg's learned correction runs on the GPU
(csrc/rtg_nn.cu), so that its features, moments, coefficients, correction,
loss and gradients can be checked against an independent implementation.
Only ``tests/`` may import it, never as the thing that is measured or shipped.

Definitions (shared with the CUDA kernels):

* a *row* is one (element e = (column C, angular cell K), spatial node ij)
  pair, rows ordered by element (global element order) and then ij = i*ny + j;
* physics features of a row (kappa, sigma at the node; h = min(dx, dy);
  c = sigma/kappa; column means are sum_ij (wx_i wy_j / 4) of the node values;
  neighbour means average over the distinct face-neighbour columns, 0 if none;
  the face mean across F averages the (up to two) neighbours there, or is the
  column's own value without one):
    [log1p(kappa h), c, -log(max(1 - c, 0) + 1e-3), log1p(max(kappa - sigma, 0) h),
     <cos>_K, <sin>_K, dth_K / 2 pi, (nx-1)/8, (nth-1)/8, free faces / 4,
     tau_C, nbr mean tau, c_C, nbr mean c, px gx + py gy, |(gx, gy)|]
  with tau_C, c_C the column means of log1p(kappa h) and c, gx = face mean of
  tau across face 0 minus across face 2, gy = face 1 minus face 3, and
  px = 2i/(nx-1) - 1, py = 2j/(ny-1) - 1 (0 for a single node);
* moments of z per row: m = [m0, m1c, m1s, phi, em, cm, nm, 0] with
    m0, m1c, m1s = sum_a w_a (1, cos th_a, sin th_a) z_a / sum_a w_a,
    phi(C, ij) = sum_K (dth_K / 2) sum_a w_a z / (2 pi),
    em(e) = sum_ij (wx wy / 4) m0,  cm(C) = sum_ij (wx wy / 4) phi,
    nm(C) = mean of cm over the distinct face-neighbour columns (0 if none);
* network: h1 = relu(F W1 + b1), h2 = relu(h1 W2 + b2),
  C = g (h2 W3 + b3) with the gate g = s / (1 + s), s = F1 (e^F0 - 1) (the
  node's sigma h), 16 -> 128 -> 128 -> 24, weights rounded to BF16; C[3][8]
  per row;
* correction: o = C m, (L z)_beta = o0 + o1 cos th_a + o2 sin th_a at unknowns;
* training statistics per row for a target error e, t = (e - z)/s with
  s = sqrt(sum z^2 / N), b_a = (1, cos th_a, sin th_a), unknown rows only:
    G = sum_a b_a b_a^T (6 entries), q = sum_a b_a t_a, c = sum_a t_a^2,
  times a weight; loss = sum_rows o^T G o - 2 q^T o + c with o = C m / s.
"""

import math

import numpy as np

from . import rt_oracle as ro

N_IN, N_HID, N_MOM, N_OUT = 16, 128, 8, 24
SHAPES = [("W1", (N_IN, N_HID)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_OUT)), ("b3", (N_OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def bf16_round(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def device_params(p):
    """The parameters the GPU runs with: weights rounded to BF16, biases FP32."""
    d = unpack(np.asarray(p, dtype=np.float32))
    for name in ("W1", "W2", "W3"):
        d[name] = bf16_round(d[name]).astype(np.float64)
    for name in ("b1", "b2", "b3"):
        d[name] = np.asarray(d[name], dtype=np.float32).astype(np.float64)
    return pack(d)


class RowLayout:
    """Rows, their elements and the per-node tables of the learned correction."""

    def __init__(self, mesh, kappa, sigma):
        L = ro.Layout(mesh)
        self.L = L
        self.mesh = mesh
        col_index = {ck: c for c, ck in enumerate(L.col_keys)}
        self.rows = []        # (elem index, i, j)
        self.elem = []        # per element: dict
        self.cols = []        # per column: dict
        for c, ck in enumerate(L.col_keys):
            col = mesh.cols[ck]
            x0, y0, x1, y1, nx, ny, tx, wx, ty, wy = ro._col_geom(col)
            xx, yy = ro.push(x0, x1, tx), ro.push(y0, y1, ty)
            kap = ro._field(kappa, xx, yy, nx, ny)
            sig = ro._field(sigma, xx, yy, nx, ny)
            nbrs = []
            faces = []
            free = 0
            for F in range(4):
                keys = col.nhbr_keys[F]
                if keys[0] is None and keys[1] is None:
                    free += 1
                faces.append([col_index[k] for k in keys if k is not None])
                for k in keys:
                    if k is not None and col_index[k] not in nbrs:
                        nbrs.append(col_index[k])
            elems = []
            for kk in sorted(col.cells.keys()):
                cell = col.cells[kk]
                nth = cell.ndofs[0]
                tb, wth = ro.lg_nodes(nth)
                th = ro.push(cell.pos[0], cell.pos[1], tb)
                e = len(self.elem)
                self.elem.append(dict(col=c, off=L.off[(ck, kk)], nth=nth, w=wth, cos=np.cos(th),
                                      sin=np.sin(th), dth=cell.pos[1] - cell.pos[0]))
                elems.append(e)
                for i in range(nx):
                    for j in range(ny):
                        self.rows.append((e, i, j))
            self.cols.append(dict(nx=nx, ny=ny, wx=wx, wy=wy, h=min(x1 - x0, y1 - y0), kap=kap, sig=sig,
                                  nbrs=nbrs, faces=faces, free=free, elems=elems))
        self.mask = ro.interior_mask(mesh, L)
        self.N = L.N

    # ------------------------------------------------------------ features
    def physics(self):
        nc = len(self.cols)
        tau_c = np.zeros(nc)
        alb_c = np.zeros(nc)
        for c, C in enumerate(self.cols):
            ww = C["wx"][:, None] * C["wy"][None, :] / 4.
            kap = np.maximum(C["kap"], 0.)
            tau_c[c] = (ww * np.log1p(kap * C["h"])).sum()
            alb = np.where(C["kap"] > 0., C["sig"] / np.where(C["kap"] > 0., C["kap"], 1.), 0.)
            alb_c[c] = (ww * alb).sum()

        def nmean(C, a):
            return np.mean([a[b] for b in C["nbrs"]]) if C["nbrs"] else 0.

        def fmean(c, F, a):
            f = self.cols[c]["faces"][F]
            return float(np.mean([a[b] for b in f])) if f else a[c]

        F = np.zeros((len(self.rows), N_IN))
        for r, (e, i, j) in enumerate(self.rows):
            E = self.elem[e]
            c = E["col"]
            C = self.cols[c]
            kap = max(C["kap"][i, j], 0.)
            sig = C["sig"][i, j]
            alb = sig / kap if kap > 0. else 0.
            sw = E["w"].sum()
            gx = fmean(c, 0, tau_c) - fmean(c, 2, tau_c)
            gy = fmean(c, 1, tau_c) - fmean(c, 3, tau_c)
            px = 2. * i / (C["nx"] - 1) - 1. if C["nx"] > 1 else 0.
            py = 2. * j / (C["ny"] - 1) - 1. if C["ny"] > 1 else 0.
            F[r] = [math.log1p(kap * C["h"]), alb, -math.log(max(1. - alb, 0.) + 1e-3),
                    math.log1p(max(kap - sig, 0.) * C["h"]),
                    (E["w"] * E["cos"]).sum() / sw, (E["w"] * E["sin"]).sum() / sw, E["dth"] / (2. * math.pi),
                    (C["nx"] - 1) / 8., (E["nth"] - 1) / 8., C["free"] / 4.,
                    tau_c[c], nmean(C, tau_c), alb_c[c], nmean(C, alb_c), px * gx + py * gy,
                    math.sqrt(gx * gx + gy * gy)]
        return F

    def moments(self, z):
        """m(z) per row (unscaled) and s = rms(z)."""
        z = np.asarray(z, dtype=np.float64)
        s = math.sqrt(float(np.dot(z, z)) / self.N)
        if not s > 0.:
            s = 1.
        nc = len(self.cols)
        mom = {}
        phi = []
        em = np.zeros(len(self.elem))
        cm = np.zeros(nc)
        for c, C in enumerate(self.cols):
            nx, ny = C["nx"], C["ny"]
            ph = np.zeros((nx, ny))
            for e in C["elems"]:
                E = self.elem[e]
                ze = z[E["off"]:E["off"] + nx * ny * E["nth"]].reshape(nx, ny, E["nth"])
                sw = E["w"].sum()
                m = (ze * E["w"]).sum(-1) / sw
                mom[e] = (m, (ze * E["w"] * E["cos"]).sum(-1) / sw, (ze * E["w"] * E["sin"]).sum(-1) / sw)
                ph += (E["dth"] / 2.) * (ze * E["w"]).sum(-1) / (2. * math.pi)
                em[e] = (C["wx"][:, None] * C["wy"][None, :] * m).sum() / 4.
            phi.append(ph)
            cm[c] = (C["wx"][:, None] * C["wy"][None, :] * ph).sum() / 4.
        nm = np.array([np.mean([cm[b] for b in C["nbrs"]]) if C["nbrs"] else 0. for C in self.cols])
        M = np.zeros((len(self.rows), N_MOM))
        for r, (e, i, j) in enumerate(self.rows):
            c = self.elem[e]["col"]
            a, b, d = mom[e]
            M[r] = [a[i, j], b[i, j], d[i, j], phi[c][i, j], em[e], cm[c], nm[c], 0.]
        return M, s

    def _row_slice(self, r):
        e, i, j = self.rows[r]
        E = self.elem[e]
        C = self.cols[E["col"]]
        o = E["off"] + (i * C["ny"] + j) * E["nth"]
        return E, slice(o, o + E["nth"])

    def correction(self, coef, z):
        """L z for per-row coefficients coef[rows][24]."""
        M, _ = self.moments(z)
        d = np.zeros(self.N)
        for r in range(len(self.rows)):
            E, sl = self._row_slice(r)
            if not self.mask[sl.start]:
                continue
            o = coef[r].reshape(3, N_MOM) @ M[r]
            d[sl] = o[0] + o[1] * E["cos"] + o[2] * E["sin"]
        return d

    def stats(self, z, e, s, weight):
        """Per-row [G00 G01 G02 G11 G12 G22 q0 q1 q2 c] times weight."""
        t = (np.asarray(e, dtype=np.float64) - np.asarray(z, dtype=np.float64)) / s
        S = np.zeros((len(self.rows), 10))
        for r in range(len(self.rows)):
            E, sl = self._row_slice(r)
            if not self.mask[sl.start]:
                continue
            B = np.stack([np.ones(E["nth"]), E["cos"], E["sin"]])
            G = B @ B.T
            q = B @ t[sl]
            S[r] = weight * np.array([G[0, 0], G[0, 1], G[0, 2], G[1, 1], G[1, 2], G[2, 2],
                                      q[0], q[1], q[2], float(t[sl] @ t[sl])])
        return S


def gate(F):
    s = np.maximum(F[:, 1] * np.expm1(F[:, 0]), 0.)
    return s / (1. + s)


def forward(p, F):
    d = unpack(p)
    a1 = F @ d["W1"] + d["b1"]
    h1 = np.maximum(a1, 0.)
    a2 = h1 @ d["W2"] + d["b2"]
    h2 = np.maximum(a2, 0.)
    o = gate(F)[:, None] * (h2 @ d["W3"] + d["b3"])
    return o, (h1, h2)


def loss_grad(p, F, M, S):
    """Loss sum_rows o^T G o - 2 q^T o + c, o = C m, and its gradient w.r.t. p."""
    d = unpack(p)
    coef, (h1, h2) = forward(p, F)
    Cm = coef.reshape(-1, 3, N_MOM)
    o = np.einsum("rkl,rl->rk", Cm, M)
    G = np.zeros((len(F), 3, 3))
    for k, a, b in [(0, 0, 0), (1, 0, 1), (2, 0, 2), (3, 1, 1), (4, 1, 2), (5, 2, 2)]:
        G[:, a, b] = S[:, k]
        G[:, b, a] = S[:, k]
    q = S[:, 6:9]
    Go = np.einsum("rab,rb->ra", G, o)
    loss = float((o * Go).sum() - 2. * (q * o).sum() + S[:, 9].sum())
    do = 2. * (Go - q)
    dcoef = gate(F)[:, None] * np.einsum("rk,rl->rkl", do, M).reshape(len(F), N_OUT)
    g = {}
    g["W3"] = h2.T @ dcoef
    g["b3"] = dcoef.sum(0)
    dh2 = (dcoef @ d["W3"].T) * (h2 > 0)
    g["W2"] = h1.T @ dh2
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ d["W2"].T) * (h1 > 0)
    g["W1"] = F.T @ dh1
    g["b1"] = dh1.sum(0)
    return loss, pack(g)


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.):
    m = b1 * m + (1. - b1) * g
    v = b2 * v + (1. - b2) * g * g
    mh = m / (1. - b1 ** step)
    vh = v / (1. - b2 ** step)
    p = p - lr * (mh / (np.sqrt(vh) + eps) + wd * p)
    return p, m, v

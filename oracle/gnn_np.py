"""ORACLE / TEST INFRASTRUCTURE ONLY -- numpy restatement of the learned
preconditioner (the message-passing network of sysu_cfd_heat_gb300/csrc/gnn.cu),
its loss, the analytic gradient and Adam, used to check the GPU kernels.  It is
never imported by the product.

The reference has no learned part (its p' solve is CG + SSOR,
navier_pressure.cpp:29); this file pins the network's definition instead:
* `exact=True`: the network in float64 without any rounding -- its analytic
  gradient is checked against central finite differences (tests/test_cpu_gnn.py);
* `exact=False`: the GPU's arithmetic -- weights, activations and the operands of
  the dense products rounded to BF16 (round to nearest even) at the points where
  the kernels round them, float32 elsewhere -- so the GPU's z, loss and gradient
  can be compared with tolerances of BF16 size.

Network, for a symmetric matrix A (diagonal d, off-diagonal part O) and residual r:
    s = rms(r / d),  u = r / (d s),  h0 = u e + c,  m^l = (O h^{l-1}) / d,
    h^l = h^{l-1} + relu([h^{l-1}, m^l] W_l + b_l),   l = 1..4,
    z = s (u + h4 w_d + b_d).
Loss of a pair (r, e = A^-1 r), S = sgn(d) A positive definite, t = z - e:
    kind 0:  t^T S t / e^T S e        kind 1:  |S t|^2 / |S e|^2
"""
from __future__ import annotations

import numpy as np

WIDTH, LAYERS = 32, 4
OFF_ENC = 0
OFF_LAYER = 64
LAYER_STRIDE = 64 * 32 + 32
OFF_DEC = OFF_LAYER + LAYERS * LAYER_STRIDE
NPARAM = OFF_DEC + 33


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return (b & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p)
    enc_e = p[OFF_ENC:OFF_ENC + 32]
    enc_c = p[OFF_ENC + 32:OFF_ENC + 64]
    Ws, bs = [], []
    for l in range(LAYERS):
        o = OFF_LAYER + l * LAYER_STRIDE
        Ws.append(p[o:o + 2048].reshape(64, 32))
        bs.append(p[o + 2048:o + 2080])
    wd = p[OFF_DEC:OFF_DEC + 32]
    bd = p[OFF_DEC + 32]
    return enc_e, enc_c, Ws, bs, wd, bd


class Graph:
    """CSR matrix split into diagonal and off-diagonal parts."""

    def __init__(self, rowptr, col, val, dtype=np.float64):
        n = len(rowptr) - 1
        self.n = n
        rows = np.repeat(np.arange(n), np.diff(rowptr))
        col = np.asarray(col)
        val = np.asarray(val, dtype=np.float64)
        diag = np.zeros(n)
        np.add.at(diag, rows[col == rows], val[col == rows])
        off = col != rows
        self.rows, self.cols, self.vals = rows[off], col[off], val[off].astype(dtype)
        self.d = diag
        self.dtype = dtype
        self.dinv = (1.0 / diag).astype(dtype)
        self.diag = diag.astype(dtype)
        self.sgn = -1.0 if diag[0] < 0 else 1.0

    def off(self, x):
        """O x (x of shape (n,) or (n, k))."""
        x = np.asarray(x)
        out = np.zeros((self.n,) + x.shape[1:], dtype=np.float64)
        contrib = self.vals.reshape((-1,) + (1,) * (x.ndim - 1)) * x[self.cols]
        np.add.at(out, self.rows, contrib)
        return out.astype(self.dtype)

    def matvec(self, x):
        return (self.off(x) + (self.diag.reshape((-1,) + (1,) * (np.ndim(x) - 1)) * x)).astype(self.dtype)


def forward(p, g: Graph, r, exact=False, skip=1.0):
    dt = np.float64 if exact else np.float32
    rnd = (lambda x: np.asarray(x, dtype=dt)) if exact else bf16
    e, c, Ws, bs, wd, bd = [np.asarray(a, dtype=dt) if np.ndim(a) else dt(a) for a in unpack(p)]
    r = np.asarray(r, dtype=dt)
    dinv = g.dinv.astype(dt)
    s = np.sqrt(np.mean((dinv.astype(np.float64) * r) ** 2))
    inv_s = dt(1.0 / s) if s > 0 else dt(0.0)
    s = dt(s)
    u = dinv * r * inv_s
    a = dinv * g.off(dinv * r).astype(dt) * inv_s
    w = dinv * g.off(np.ones(g.n, dtype=dt)).astype(dt)
    h = rnd(u[:, None] * e + c)
    m = rnd(a[:, None] * e + w[:, None] * c)
    cache = {"s": s, "u": u, "a": a, "w": w, "X": [], "pre": [], "h": [h]}
    for l in range(LAYERS):
        if l > 0:
            m = rnd(dinv[:, None] * g.off(h).astype(dt))
        X = np.concatenate([h, m], axis=1)
        pre = (X.astype(np.float64) @ rnd(Ws[l]).astype(np.float64)).astype(dt) + bs[l]
        h = rnd(h + np.maximum(pre, 0))
        cache["X"].append(X)
        cache["pre"].append(pre)
        cache["h"].append(h)
    z = s * (dt(skip) * u + (h.astype(np.float64) @ wd.astype(np.float64)).astype(dt) + bd)
    return z.astype(dt), cache


def loss_and_grad(p, g: Graph, r, e_true, kind=0, exact=False, skip=1.0):
    """Loss of one pair and its gradient with respect to the flat parameters."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda x: np.asarray(x, dtype=dt)) if exact else bf16
    z, C = forward(p, g, r, exact, skip)
    e_true = np.asarray(e_true, dtype=dt)
    t = z - e_true
    St = g.sgn * g.matvec(t).astype(np.float64)
    Se = g.sgn * g.matvec(e_true).astype(np.float64)
    if kind == 0:
        num = float(t.astype(np.float64) @ St)
        den = float(e_true.astype(np.float64) @ Se)
        gz = 2.0 * St / den
    else:
        num = float(St @ St)
        den = float(Se @ Se)
        gz = 2.0 * g.sgn * g.matvec(St).astype(np.float64) / den
    loss = num / den
    enc_e, enc_c, Ws, bs, wd, bd = unpack(p)
    grad = np.zeros(NPARAM)
    s = float(C["s"])
    gs = gz * s
    h4 = C["h"][LAYERS].astype(np.float64)
    grad[OFF_DEC:OFF_DEC + 32] = gs @ h4
    grad[OFF_DEC + 32] = gs.sum()
    delta = gs[:, None] * np.asarray(wd, dtype=np.float64)[None, :]
    dinv = g.dinv.astype(np.float64)
    for l in reversed(range(LAYERS)):
        mask = C["pre"][l] > 0
        dpre = rnd(np.where(mask, delta, 0.0).astype(dt)).astype(np.float64)
        X = C["X"][l].astype(np.float64)
        o = OFF_LAYER + l * LAYER_STRIDE
        grad[o:o + 2048] = (X.T @ dpre).reshape(-1)
        grad[o + 2048:o + 2080] = dpre.sum(axis=0)
        dX = dpre @ rnd(np.asarray(Ws[l], dtype=dt)).astype(np.float64).T
        dxh, dxm = dX[:, :32], dX[:, 32:]
        if l > 0:
            delta = delta + dxh + g.off(dinv[:, None] * dxm).astype(np.float64)
        else:
            dh0 = delta + dxh
            u, a, w = (C[k].astype(np.float64) for k in ("u", "a", "w"))
            grad[OFF_ENC:OFF_ENC + 32] = u @ dh0 + a @ dxm
            grad[OFF_ENC + 32:OFF_ENC + 64] = dh0.sum(axis=0) + w @ dxm
    return loss, grad, z


def loss_only(p, g: Graph, r, e_true, kind=0):
    z, _ = forward(p, g, r, exact=True)
    t = z - e_true
    St = g.sgn * g.matvec(t)
    Se = g.sgn * g.matvec(e_true)
    if kind == 0:
        return float(t @ St) / float(e_true @ Se)
    return float(St @ St) / float(Se @ Se)


def init_params(seed=0):
    """Same distribution as the library's sysu_gnn_init_params (not the same draws)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)
    p[OFF_ENC:OFF_ENC + 64] = rng.uniform(-1, 1, 64)
    a = np.sqrt(6.0 / 96.0) * 0.5
    for l in range(LAYERS):
        o = OFF_LAYER + l * LAYER_STRIDE
        p[o:o + 2048] = rng.uniform(-a, a, 2048)
    return p


def laplacian_3d(nx, ny, nz, seed=0, jitter=0.3, negative=True):
    """A p'-like test matrix: 7-point finite-volume Laplacian on an nx x ny x nz
    grid with random positive face coefficients (1 +- jitter), Dirichlet-like
    boundary rows strengthened so the matrix is definite; negative diagonal like
    the reference's p' matrix (navier_pressure.cpp:150-163) when `negative`."""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    idx = np.arange(n).reshape(nx, ny, nz)
    rows, cols, vals = [], [], []
    diag = np.zeros(n)
    for ax in range(3):
        a = np.take(idx, range(0, idx.shape[ax] - 1), axis=ax).ravel()
        b = np.take(idx, range(1, idx.shape[ax]), axis=ax).ravel()
        cf = 1.0 + jitter * rng.uniform(-1, 1, len(a))
        rows += [a, b]
        cols += [b, a]
        vals += [cf, cf]
        np.add.at(diag, a, cf)
        np.add.at(diag, b, cf)
    boundary = np.zeros(n, bool)
    for ax in range(3):
        boundary |= (np.indices((nx, ny, nz))[ax] == 0).ravel()
    diag[boundary] += 1.0
    rows = np.concatenate(rows + [np.arange(n)])
    cols = np.concatenate(cols + [np.arange(n)])
    vals = np.concatenate([-v for v in vals] + [diag])
    if negative:
        vals = -vals
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, cols.astype(np.int32), vals

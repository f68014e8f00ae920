"""The learned preconditioner's oracle (oracle/gnn_np.py) on the CPU: its analytic
gradient against central finite differences, its BF16 rounding, and the
network's reduction to the Jacobi preconditioner at zero decoder weights."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import gnn_np as G  # noqa: E402


def _case(seed=0, n=(5, 4, 3)):
    rp, cl, vl = G.laplacian_3d(*n, seed=seed)
    g = G.Graph(rp, cl, vl)
    rng = np.random.default_rng(seed + 1)
    r = rng.standard_normal(g.n)
    A = np.zeros((g.n, g.n))
    rows = np.repeat(np.arange(g.n), np.diff(rp))
    A[rows, cl] = vl
    e = np.linalg.solve(A, r)
    return g, r, e, A


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e38, 1.0 + 2.0 ** -9], np.float32)
    got = G.bf16(x)
    want = np.array([1.0, 1.0, 1.0 + 2.0 ** -6, -2.5, 2.9999e38, 1.0], np.float32)
    assert got[0] == 1.0 and got[1] == 1.0          # tie -> even
    assert got[2] == np.float32(1.0 + 2.0 ** -6)     # tie -> even (up)
    assert got[3] == -2.5 and got[5] == 1.0
    assert abs(got[4] / want[4] - 1) < 1e-2


def test_zero_decoder_is_jacobi():
    g, r, e, _ = _case()
    p = G.init_params(3).astype(np.float64)
    for exact in (True, False):
        z, _ = G.forward(p, g, r, exact=exact)
        np.testing.assert_allclose(z, r / g.d, rtol=1e-6 if not exact else 1e-14)


@pytest.mark.parametrize("kind", [0, 1])
def test_gradient_matches_finite_differences(kind):
    g, r, e, _ = _case(seed=4)
    rng = np.random.default_rng(7)
    p = G.init_params(5).astype(np.float64)
    p[G.OFF_DEC:G.OFF_DEC + 33] = rng.uniform(-0.5, 0.5, 33)
    for l in range(G.LAYERS):
        o = G.OFF_LAYER + l * G.LAYER_STRIDE
        p[o + 2048:o + 2080] = rng.uniform(-0.2, 0.2, 32)
    loss, grad, _ = G.loss_and_grad(p, g, r, e, kind=kind, exact=True)
    assert abs(loss - G.loss_only(p, g, r, e, kind)) < 1e-12 * max(1.0, loss)
    idx = np.concatenate([rng.choice(np.arange(G.OFF_ENC, G.OFF_ENC + 64), 8, replace=False),
                          rng.choice(np.arange(G.OFF_LAYER, G.OFF_DEC), 40, replace=False),
                          rng.choice(np.arange(G.OFF_DEC, G.NPARAM), 6, replace=False)])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (G.loss_only(pp, g, r, e, kind) - G.loss_only(pm, g, r, e, kind)) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-5 * max(1e-3, abs(grad[k]), abs(fd)), (k, fd, grad[k])


def test_bf16_forward_close_to_exact():
    g, r, e, _ = _case(seed=9)
    p = G.init_params(2).astype(np.float64)
    p[G.OFF_DEC:G.OFF_DEC + 32] = np.random.default_rng(1).uniform(-0.3, 0.3, 32)
    z0, _ = G.forward(p, g, r, exact=True)
    z1, _ = G.forward(p, g, r, exact=False)
    assert np.linalg.norm(z1 - z0) / np.linalg.norm(z0) < 2e-2

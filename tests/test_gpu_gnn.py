"""Learned preconditioner on the GPU against its oracle (oracle/gnn_np.py):
network output, hidden states, loss and gradient (BF16 tolerances), training,
and flexible CG with the network -- fewer iterations than without it, the same
FP64 stopping test, and the Jacobi fallback when the network is useless."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import gnn_np as G  # noqa: E402

from sysu_cfd_heat_gb300.learned import LearnedPreconditioner  # noqa: E402

pytestmark = pytest.mark.gpu


def _params(seed):
    rng = np.random.default_rng(seed)
    p = G.init_params(seed)
    p[G.OFF_DEC:G.OFF_DEC + 33] = rng.uniform(-0.3, 0.3, 33)
    for l in range(G.LAYERS):
        o = G.OFF_LAYER + l * G.LAYER_STRIDE
        p[o + 2048:o + 2080] = rng.uniform(-0.1, 0.1, 32)
    return p


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("shape", [(4, 4, 5), (10, 10, 13), (40, 40, 40)])
def test_forward_matches_oracle(shape):
    rp, cl, vl = G.laplacian_3d(*shape, seed=1)
    g = G.Graph(rp, cl, vl)
    r = np.random.default_rng(2).standard_normal(g.n)
    p = _params(3)
    with LearnedPreconditioner(rp, cl, vl) as net:
        net.params = p
        assert np.array_equal(net.params, p)
        _, cache = G.forward(p, g, r, exact=False)
        errs = [_rel(net.hidden(r, l), cache["h"][l]) for l in range(1, 5)]
        z = net.apply(r)
        zo, _ = G.forward(p, g, r, exact=False)
        assert max(errs) < 5e-3, errs
        assert _rel(z, zo) < 5e-3, (_rel(z, zo), errs)
        # zero decoder: exactly Jacobi (up to the FP32 output)
        q = p.copy()
        q[G.OFF_DEC:] = 0
        net.params = q
        assert _rel(net.apply(r), r / g.d) < 1e-6


@pytest.mark.parametrize("kind", [0, 1])
def test_loss_and_gradient_match_oracle(kind):
    rp, cl, vl = G.laplacian_3d(12, 10, 9, seed=5)
    g = G.Graph(rp, cl, vl)
    rng = np.random.default_rng(6)
    r = rng.standard_normal(g.n)
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    A = sp.csr_matrix((vl, cl, rp), shape=(g.n, g.n))
    e = spl.spsolve(A.tocsc(), r)
    p = _params(8)
    lo, go, _ = G.loss_and_grad(p, g, r, e, kind=kind, exact=False)
    with LearnedPreconditioner(rp, cl, vl) as net:
        net.params = p
        net.add_pair(r, e)
        loss, grad = net.loss_grad(0, kind)
    assert abs(loss - lo) <= 2e-3 * abs(lo), (loss, lo)
    blocks = {"enc": slice(G.OFF_ENC, G.OFF_ENC + 64), "dec": slice(G.OFF_DEC, G.NPARAM)}
    for l in range(G.LAYERS):
        o = G.OFF_LAYER + l * G.LAYER_STRIDE
        blocks[f"W{l}"] = slice(o, o + 2048)
        blocks[f"b{l}"] = slice(o + 2048, o + 2080)
    errs = {k: _rel(grad[s], go[s]) for k, s in blocks.items()}
    assert max(errs.values()) < 2e-2, errs


def _p_system(shape=(24, 24, 24), seed=11):
    rp, cl, vl = G.laplacian_3d(*shape, seed=seed, jitter=0.5)
    n = len(rp) - 1
    return rp, cl, vl, n


def _solve_pairs(net, rp, cl, vl, n, count, seed):
    """Residual/correction pairs from partial solves, as the SIMPLE loop makes them."""
    rng = np.random.default_rng(seed)
    for k in range(count):
        b = rng.standard_normal(n)
        x, info = net.fcg(b, eps=1e-10, use_gnn=False)
        assert info["status"] == 0
        net.add_pair(b, x)
        x1, _ = net.fcg(b, eps=10.0 ** -(1 + k % 3), use_gnn=False, inner_tol=0.5)
        import scipy.sparse as sp
        A = sp.csr_matrix((vl, cl, rp), shape=(n, n))
        net.add_pair(b - A @ x1, x - x1)


def test_training_reduces_loss_and_fcg_iterations():
    rp, cl, vl, n = _p_system()
    with LearnedPreconditioner(rp, cl, vl, capacity=24) as net:
        net.init_params(1)
        _solve_pairs(net, rp, cl, vl, n, 12, 3)
        b = np.random.default_rng(99).standard_normal(n)
        _, jac = net.fcg(b, eps=1e-8, use_gnn=False)
        _, init = net.fcg(b, eps=1e-8, use_gnn=True)
        # zero decoder at init: the network is Jacobi
        assert abs(init["iters"] - jac["iters"]) <= 2, (init, jac)
        losses = net.train(600, lr=2e-3)
        assert np.all(np.isfinite(losses))
        first, last = losses[:24].mean(), losses[-24:].mean()
        assert last < 0.9 * first, (first, last)
        x, tr = net.fcg(b, eps=1e-8, use_gnn=True)
        assert tr["status"] == 0 and tr["res"] < 1e-8 and tr["fallback_at"] == -1, tr
        import scipy.sparse as sp
        A = sp.csr_matrix((vl, cl, rp), shape=(n, n))
        assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-8
        # the gain: fewer iterations than the same flexible CG with Jacobi
        assert tr["iters"] < 0.8 * jac["iters"], (tr, jac)


def test_fallback_when_network_is_useless():
    rp, cl, vl, n = _p_system((16, 16, 16), 4)
    rng = np.random.default_rng(0)
    p = G.init_params(0)
    p[G.OFF_DEC:G.OFF_DEC + 33] = rng.uniform(-50, 50, 33)  # a decoder that wrecks the direction
    b = rng.standard_normal(n)
    with LearnedPreconditioner(rp, cl, vl) as net:
        net.params = p
        x, info = net.fcg(b, eps=1e-8, use_gnn=True, stall_max=10)
        _, jac = net.fcg(b, eps=1e-8, use_gnn=False)
    assert info["status"] == 0 and info["res"] < 1e-8
    assert info["fallback_at"] >= 0
    import scipy.sparse as sp
    A = sp.csr_matrix((vl, cl, rp), shape=(n, n))
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-8
    assert jac["fallback_at"] == -1


def test_fcg_jacobi_matches_cg():
    """Flexible CG with Jacobi and FP32 recurrences converges like Jacobi-CG."""
    from sysu_cfd_heat_gb300 import _lib
    import ctypes as C
    rp, cl, vl, n = _p_system((20, 20, 20), 2)
    b = np.random.default_rng(5).standard_normal(n)
    with LearnedPreconditioner(rp, cl, vl) as net:
        x, info = net.fcg(b, eps=1e-10, use_gnn=False)
    L = _lib.lib()
    xc = np.zeros(n)
    it, res, st = C.c_int(), C.c_double(), C.c_int()
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    assert L.sysu_csr_solve(0, 1, n, ip(rp), ip(cl), dp(vl), dp(b), dp(xc), 5000, 1e-10, 1.0, C.byref(it),
                            C.byref(res), C.byref(st)) == 0
    assert info["status"] == 0 and info["res"] < 1e-10
    assert abs(info["iters"] - it.value) <= 0.1 * it.value + 5, (info, it.value)
    assert _rel(x, xc) < 1e-8


def test_simple_learned_form_matches_fp64():
    """The SIMPLE loop with the learned p' form (option p.learned): fields after
    30 outer iterations within 1e-6 of the plain FP64 form, every p' solve to
    its tolerance, fewer p' iterations once trained."""
    import tempfile
    from sysu_cfd_heat_gb300 import meshgen as mg
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    with tempfile.TemporaryDirectory() as d:
        p = mg.write_case(d, mg.lid_cavity_tet(12, 12, 8, jitter=0.2, seed=7), mg.cavity_param("x", 100, mu=0.0025))
        out = {}
        for name, opts in (("fp64", {}), ("learned", {"p.learned": 1, "p.learn_iters": 8, "p.learn_steps": 48})):
            o = {"rtc": 1e-10, "p.maxit": 20000}
            o.update(opts)
            with NavierStokesSolver(p, o) as s:
                its = []
                for k in range(30):
                    assert s.iterate(1) == 1
                    st = s.solve_stats()["p"]
                    assert st["status"][0] == 0 and st["res"][0] < 1e-10, (name, k, st)
                    its.append(st["iters"][0])
                out[name] = ({f: s.get(f) for f in ("U", "V", "W", "P")}, its)
                if name == "learned":
                    assert s.get_option("p.learned_solves") == 30
    for f, a in out["fp64"][0].items():
        assert _rel(out["learned"][0][f], a) < 1e-6, f
    assert np.mean(out["learned"][1][-10:]) < 0.8 * np.mean(out["fp64"][1][-10:]), (out["learned"][1], out["fp64"][1])

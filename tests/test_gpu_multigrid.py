"""The aggregation-multigrid forms of the p' solve on the GPU.

* one application of the cycle (FP32) against the numpy oracle (oracle/amg_np.py,
  FP64), with the Jacobi post-smoother and with the network as post-smoother
  (oracle/gnn_np.py for the network, BF16 tolerance);
* the multigrid flexible CG (CSR method 5): same stopping test as every solve,
  solutions equal to the FP64 CG's, a fraction of its iterations, on singular
  (pure-Neumann) and definite systems;
* the SIMPLE loop with p' option precond 4: fields equal to the plain FP64
  form's when both solve tightly;
* the learned form: the network trained on the solver's own pairs (turned into
  post-smoother pairs) needs fewer iterations than the same cycle with the
  untrained network, and a useless network falls back to the Jacobi
  post-smoother and still converges -- with the network at the finest level
  (CSR handle) and on a coarse level of the SIMPLE p' solve (option
  p.learn_level), where the untrained network is exactly the plain cycle.
"""
import os
import sys
import tempfile

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import amg_np  # noqa: E402
import gnn_np as G  # noqa: E402
from sysu_cfd_heat_gb300 import meshgen as mg  # noqa: E402
from sysu_cfd_heat_gb300.learned import LearnedPreconditioner  # noqa: E402
from sysu_cfd_heat_gb300.solver import NavierStokesSolver, csr_solve  # noqa: E402

pytestmark = pytest.mark.gpu
DENSE_MAX = 200  # the library's coarsest dense level


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _mean_free(x):
    return x - x.mean()


@pytest.mark.parametrize("kind,shape", [("neumann", (22, 20, 18)), ("dirichlet", (17, 15, 13)),
                                        ("dirichlet", (5, 5, 4))])
def test_cycle_matches_oracle(kind, shape):
    if kind == "neumann":
        rp, cl, vl = amg_np.neumann_3d(*shape, seed=7)
    else:
        rp, cl, vl = G.laplacian_3d(*shape, seed=7)
    lv = amg_np.hierarchy(rp, cl, vl, dense_max=DENSE_MAX)
    r = np.random.default_rng(8).standard_normal(lv[0].n)
    if kind == "neumann":
        r -= r.mean()
    with LearnedPreconditioner(rp, cl, vl) as net:
        rows = net.set_multigrid()
        assert rows == [L.n for L in lv], (rows, [L.n for L in lv])
        z = net.mg_apply(r, use_gnn=False)
    zo = amg_np.vcycle(lv, r)
    assert _rel(z, zo) < 5e-5, _rel(z, zo)


def test_cycle_with_network_post_smoother_matches_oracle():
    rp, cl, vl = G.laplacian_3d(20, 18, 16, seed=3)
    lv = amg_np.hierarchy(rp, cl, vl, dense_max=DENSE_MAX)
    r = np.random.default_rng(4).standard_normal(lv[0].n)
    rng = np.random.default_rng(5)
    p = G.init_params(5)
    p[G.OFF_DEC:G.OFF_DEC + 33] = rng.uniform(-0.3, 0.3, 33)
    with LearnedPreconditioner(rp, cl, vl) as net:
        net.params = p
        net.set_multigrid()
        z = net.mg_apply(r, use_gnn=True)
        zj = net.mg_apply(r, use_gnn=False)
    z2, t = amg_np.cycle_fixed(lv, r)
    zn, _ = G.forward(p, G.Graph(rp, cl, vl), t, exact=False, skip=0.8)
    zo = z2 + zn
    assert _rel(z, zo) < 5e-3, _rel(z, zo)
    assert _rel(zj, amg_np.vcycle(lv, r)) < 5e-5


@pytest.mark.parametrize("kind,shape", [("neumann", (40, 36, 30)), ("dirichlet", (32, 30, 28))])
def test_multigrid_cg_converges_to_the_fp64_solution(kind, shape):
    if kind == "neumann":
        rp, cl, vl = amg_np.neumann_3d(*shape, seed=9)
    else:
        rp, cl, vl = G.laplacian_3d(*shape, seed=9, jitter=0.5)
    n = len(rp) - 1
    b = np.random.default_rng(10).standard_normal(n)
    if kind == "neumann":
        b -= b.mean()  # consistent
    eps = 1e-10
    x, it, res, st = csr_solve(rp, cl, vl, b, None, method="CG-multigrid", maxit=1000, eps=eps, omega=0.8)
    xc, itc, resc, stc = csr_solve(rp, cl, vl, b, None, method="CG", precond="Jacobi", maxit=20000, eps=eps)
    assert st == 0 and stc == 0, (st, stc)
    assert res < eps
    A = sp.csr_matrix((vl, cl, rp), shape=(n, n))
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 2 * eps
    assert _rel(_mean_free(x), _mean_free(xc)) < 1e-7
    assert it * 4 < itc, (it, itc)


def test_simple_multigrid_form_matches_fp64():
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_tet(12, 12, 8, jitter=0.2), mg.cavity_param("x", 30, mu=0.0025))
        out = {}
        for name, opts in (("fp64", {}), ("multigrid", {"p.precond": 4})):
            with NavierStokesSolver(p, dict({"rtc": 1e-11, "p.maxit": 100000}, **opts)) as s:
                assert s.iterate(12) == 12
                st = s.solve_stats()["p"]
                assert st["status"][0] == 0, st
                out[name] = ({f: s.get(f) for f in ("U", "V", "W", "P")}, st["iters"][0])
        for f, a in out["multigrid"][0].items():
            assert _rel(a, out["fp64"][0][f]) < 1e-8, (f, _rel(a, out["fp64"][0][f]))
        assert out["multigrid"][1] * 5 < out["fp64"][1], (out["multigrid"][1], out["fp64"][1])


def _tet_p_systems(k=6):
    """p' systems (matrix, right-hand side) of successive outer iterations of a
    jittered-tet cavity, as the solver assembled them."""
    systems = []
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_tet(18, 18, 12, jitter=0.2, seed=5), mg.cavity_param("x", 100, mu=0.0025))
        with NavierStokesSolver(p, {"rtc": 1e-8, "p.maxit": 100000}) as s:
            for _ in range(k):
                s.CalculateVelocity()
                s.CalculatePressure()
                s.check()
                rp, cl, vl = s.matrix("p")
                systems.append((rp, cl, vl, s.get("bp")))
    return systems


def test_finest_level_network_post_smoother_trains_and_converges():
    systems = _tet_p_systems()
    rp, cl, vl, _ = systems[-1]
    n = len(rp) - 1
    with LearnedPreconditioner(rp, cl, vl, capacity=16) as net:
        net.init_params(1)
        net.set_multigrid()
        # pairs from the solves of the earlier outer iterations, as the SIMPLE loop makes them
        for rpk, clk, vlk, bk in systems[:-1]:
            net.set_values(vlk)
            x, info = net.fcg(bk, eps=1e-10, use_gnn=False)
            assert info["status"] == 0
            net.add_pair(bk, x)
            x1, _ = net.fcg(bk, eps=1e-2, use_gnn=False)
            A = sp.csr_matrix((vlk, clk, rpk), shape=(n, n))
            net.add_pair(bk - A @ x1, x - x1)
        net.set_values(vl)
        b = systems[-1][3]
        _, plain = net.fcg(b, eps=1e-8, use_gnn=False)
        _, init = net.fcg(b, eps=1e-8, use_gnn=True)
        losses = net.train(400, lr=1e-3, loss_kind=1)
        assert np.all(np.isfinite(losses))
        assert losses[-20:].mean() < 0.8 * losses[:20].mean(), (losses[:20].mean(), losses[-20:].mean())
        x, tr = net.fcg(b, eps=1e-8, use_gnn=True)
    A = sp.csr_matrix((vl, cl, rp), shape=(n, n))
    assert tr["status"] == 0 and tr["res"] < 1e-8 and tr["fallback_at"] == -1, tr
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-8
    # zero decoder at init: the network post-smoother is the cycle's Jacobi step
    assert init["fallback_at"] == -1
    assert abs(init["iters"] - plain["iters"]) <= 1, (init, plain)
    # at the finest level the trained network does not cost iterations (its gain
    # is shown on a coarse level, test_coarse_level_network_gains_over_the_plain_cycle)
    assert tr["iters"] <= init["iters"] + 2, (tr, init, plain)
    print("multigrid FCG iterations: Jacobi post-smoother", plain["iters"], "untrained network", init["iters"],
          "trained network", tr["iters"])


def test_useless_network_falls_back_to_the_jacobi_post_smoother():
    rp, cl, vl = amg_np.neumann_3d(24, 22, 20, seed=2)
    n = len(rp) - 1
    rng = np.random.default_rng(0)
    b = rng.standard_normal(n)
    b -= b.mean()
    p = G.init_params(0)
    p[G.OFF_DEC:G.OFF_DEC + 33] = rng.uniform(-50, 50, 33)
    with LearnedPreconditioner(rp, cl, vl) as net:
        net.params = p
        net.set_multigrid()
        x, info = net.fcg(b, eps=1e-8, use_gnn=True, stall_max=5)
        _, plain = net.fcg(b, eps=1e-8, use_gnn=False)
    assert info["status"] == 0 and info["res"] < 1e-8, info
    assert info["fallback_at"] >= 0
    A = sp.csr_matrix((vl, cl, rp), shape=(n, n))
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-8
    assert plain["fallback_at"] == -1 and plain["status"] == 0


def _learned_cavity(tmp, level, learn_iters=6, steps=64):
    p = mg.write_case(tmp, mg.lid_cavity_tet(18, 18, 12, jitter=0.2, seed=5), mg.cavity_param("x", 100, mu=0.0025))
    s = NavierStokesSolver(p, {"rtc": 1e-8, "p.maxit": 100000, "p.precond": 4, "p.learned": 1, "p.learn_level": level,
                               "p.learn_iters": learn_iters, "p.learn_steps": steps})
    return s


@pytest.mark.parametrize("level", [1, 2])
def test_coarse_level_network_cycle_matches_oracle(level):
    with tempfile.TemporaryDirectory() as tmp:
        with _learned_cavity(tmp, level, learn_iters=1, steps=8) as s:
            # one outer iteration: its p' solve (a training solve) set the hierarchy
            # up from this matrix -- the aggregates are fixed at the first solve and
            # later solves only refresh the values
            s.iterate(1)
            lvl, prm = s.p_network()
            assert lvl == level
            rng = np.random.default_rng(6)
            prm = prm.copy()
            prm[G.OFF_DEC:G.OFF_DEC + 33] = rng.uniform(-0.3, 0.3, 33)  # make the network's part visible
            s.p_set_network(prm)
            rp, cl, vl = s.matrix("p")
            r = rng.standard_normal(len(rp) - 1)
            r -= r.mean()
            z = s.p_cycle(r, use_net=True)
            zj = s.p_cycle(r, use_net=False)
    lv = amg_np.hierarchy(rp, cl, vl, dense_max=DENSE_MAX)
    L = lv[level]
    g = G.Graph(L.rp, L.col, L.val)

    def post(rl, zp):
        zn, _ = G.forward(prm, g, rl - L.matvec(zp), exact=False, skip=0.8)
        return zp + zn
    zo = amg_np.vcycle(lv, r, post={level: post})
    assert _rel(zj, amg_np.vcycle(lv, r)) < 5e-5
    assert _rel(z, zo) < 5e-3, _rel(z, zo)
    assert _rel(z, zj) > 1e-3  # the network did change the cycle


def test_coarse_level_network_gains_over_the_plain_cycle():
    """Trained during the first outer iterations (pairs: the right-hand sides the
    cycle hands the network's level, solved on that level), the network cuts the
    p' iterations below the plain cycle's from the same state; with its zero
    decoder the untrained network is the plain cycle."""
    fields = ("U", "V", "W", "P", "RUFace")
    with tempfile.TemporaryDirectory() as tmp:
        with _learned_cavity(tmp, 1) as s:
            assert s.iterate(6) == 6
            state = {f: s.get(f) for f in fields}
            its = {}
            for name, opts in (("plain", {"p.learned": 0}), ("trained", {"p.learned": 1}),
                               ("untrained", {"p.learned": 1, "p.learn_reset": 1, "p.learn_iters": 0})):
                for k, v in opts.items():
                    s.set_option(k, v)
                for f, a in state.items():
                    s.set(f, a)
                s.CalculateVelocity()
                s.CalculatePressure()
                s.check()
                st = s.solve_stats()["p"]
                assert st["status"][0] == 0 and st["res"][0] < 1e-8, (name, st)
                its[name] = st["iters"][0]
    assert abs(its["untrained"] - its["plain"]) <= 1, its
    assert its["trained"] < its["plain"], its
    print("p' iterations from the same state:", its)


def test_useless_coarse_level_network_still_converges():
    with tempfile.TemporaryDirectory() as tmp:
        with _learned_cavity(tmp, 1, learn_iters=1, steps=4) as s:
            s.iterate(2)
            _, prm = s.p_network()
            prm = prm.copy()
            prm[G.OFF_DEC:G.OFF_DEC + 33] = np.random.default_rng(0).uniform(-50, 50, 33)
            s.p_set_network(prm)
            s.CalculateVelocity()
            s.CalculatePressure()
            s.check()
            st = s.solve_stats()["p"]
    assert st["status"][0] == 0 and st["res"][0] < 1e-8, st


def test_host_driven_loops_give_the_same_fields():
    """Option graph_loops 0 (the host drives the multigrid FCG and mixed momentum
    iterations, as per-kernel profiling needs) runs the same kernels as the device
    loops (graph WHILE nodes): bit-identical fields and the same iteration counts."""
    import tempfile

    from sysu_cfd_heat_gb300 import meshgen as mg
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_tet(9, 8, 7, jitter=0.2), mg.cavity_param("x", 20, mu=0.0025))
        out = {}
        for loops in (1, 0):
            opts = {"rtc": 1e-8, "p.precond": 4, "p.maxit": 5000, "mom.mixed": 1, "graph_loops": loops}
            with NavierStokesSolver(p, opts) as s:
                assert s.iterate(5) == 5
                st = s.solve_stats()
                out[loops] = ({f: s.get(f) for f in ("U", "V", "W", "P")}, st["p"]["iters"][0], st["mom"]["iters"])
    for f in ("U", "V", "W", "P"):
        assert np.array_equal(out[0][0][f], out[1][0][f]), f
    assert out[0][1] == out[1][1] and out[0][2] == out[1][2]

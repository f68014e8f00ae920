"""Many cases in one CUDA graph (sysu_batch_*): the graph replays give exactly the
fields of each case run alone with the same SM cap, the autotuner's caps fit the
GPU, and the reference's convergence checks pass on every case."""
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.batch import CaseBatch
from sysu_cfd_heat_gb300.solver import NavierStokesSolver

pytestmark = pytest.mark.gpu
OPTS = {"rtc": 1e-8, "p.mixed": 1, "p.maxit": 5000}


def _cases(d, spec):
    out = []
    for k, (L, re) in enumerate(spec):
        sub = f"{d}/c{k}"
        out.append(mg.write_case(sub, mg.lid_cavity_hex(L), mg.cavity_param("x", 1000, mu=1.0 / re)))
    return out


def test_graph_replay_equals_cases_alone():
    spec = [(6, 100.0), (11, 400.0), (14, 900.0), (9, 50.0)]
    iters = 12
    with tempfile.TemporaryDirectory() as d:
        params = _cases(d, spec)
        with CaseBatch(params, OPTS) as b:
            t = b.tune((1, 2, 4, 8))
            assert sum(t["sm_cap"]) <= 152 and all(c >= 1 for c in t["sm_cap"])
            b.capture()
            b.replay(iters)
            b.check()
            got = [{f: s.get(f) for f in ("U", "V", "W", "P")} for s in b.cases]
            caps = t["sm_cap"]
        for k, p in enumerate(params):
            with NavierStokesSolver(p, dict(OPTS, sm_cap=caps[k])) as s:
                assert s.iterate(iters) == iters
                for f in ("U", "V", "W", "P"):
                    assert np.array_equal(s.get(f), got[k][f]), (k, f)
            with NavierStokesSolver(p, OPTS) as s:  # no cap: other grids, same solution
                s.iterate(iters)
                for f in ("U", "V", "W", "P"):
                    a = s.get(f)
                    assert np.linalg.norm(a - got[k][f]) <= 1e-7 * np.linalg.norm(a) + 1e-14, (k, f)


def test_graph_replay_with_mixed_momentum():
    """Option mom.mixed inside a captured outer iteration: the momentum solve's
    iterations are a WHILE node of the batch's graph (no host round trip); the
    fields equal those of each case alone with the same SM cap, and stay within the
    solve tolerance of the unbatched mixed form (u, v, w one after another)."""
    spec = [(6, 100.0), (9, 400.0)]
    iters = 8
    opts = dict(OPTS, **{"mom.mixed": 1})
    with tempfile.TemporaryDirectory() as d:
        params = _cases(d, spec)
        with CaseBatch(params, opts) as b:
            b.set_caps([2, 4])
            b.capture()
            b.replay(iters)
            b.check()
            got = [{f: s.get(f) for f in ("U", "V", "W", "P")} for s in b.cases]
            for s in b.cases:
                st = s.solve_stats()["mom"]
                assert st["status"] == [0, 0, 0] and min(st["iters"]) > 0, st
        for k, p in enumerate(params):
            with NavierStokesSolver(p, dict(opts, sm_cap=[2, 4][k])) as s:
                assert s.iterate(iters) == iters
                for f in ("U", "V", "W", "P"):
                    assert np.array_equal(s.get(f), got[k][f]), (k, f)
            with NavierStokesSolver(p, dict(opts, mom_batched=0)) as s:
                s.iterate(iters)
                for f in ("U", "V", "W", "P"):
                    a = s.get(f)
                    assert np.linalg.norm(a - got[k][f]) <= 1e-6 * np.linalg.norm(a) + 1e-14, (k, f)


def test_graph_replay_with_multigrid_pressure():
    """p' by the multigrid flexible CG (option p.precond 4) and mixed momentum inside
    the batch's graph: both solves loop on the device (WHILE nodes), the hierarchy is
    built in the eager iteration before the capture; the fields equal those of each
    case alone with the same SM cap."""
    spec = [(7, 100.0), (10, 400.0), (12, 900.0)]
    iters = 6
    opts = dict(OPTS, **{"mom.mixed": 1, "p.precond": 4, "p.mixed": 0})
    with tempfile.TemporaryDirectory() as d:
        params = _cases(d, spec)
        caps = [2, 4, 2]
        with CaseBatch(params, opts) as b:
            b.set_caps(caps)
            b.capture()
            b.replay(iters)
            b.check()
            got = [{f: s.get(f) for f in ("U", "V", "W", "P")} for s in b.cases]
            for s in b.cases:
                st = s.solve_stats()
                assert st["p"]["status"][0] == 0 and st["p"]["iters"][0] > 0, st["p"]
                assert st["mom"]["status"] == [0, 0, 0], st["mom"]
        for k, p in enumerate(params):
            with NavierStokesSolver(p, dict(opts, sm_cap=caps[k])) as s:
                assert s.iterate(iters) == iters
                for f in ("U", "V", "W", "P"):
                    assert np.array_equal(s.get(f), got[k][f]), (k, f)

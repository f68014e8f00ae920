"""Batched forms on the GPU: three same-pattern systems in one BiCGSTAB launch
(sysu_csr_bicgstab_batched3) against three single solves, and the SIMPLE loop
with option scalars_batched (k, eps, T solved together) reaching the same
steady solution as the sequential form."""
import ctypes as C
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import _lib
from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.solver import NavierStokesSolver, csr_solve

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _pattern(n, seed):
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for i in range(n):
        nb = {i} | set(rng.choice(n, 5, replace=False).tolist())
        for j in sorted(nb):
            rows.append(i)
            cols.append(j)
    rows, cols = np.array(rows), np.array(cols)
    rp = np.zeros(n + 1, np.int32)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols.astype(np.int32), rows


def test_batched3_matches_single_solves():
    n = 3000
    rp, cl, rows = _pattern(n, 1)
    rng = np.random.default_rng(2)
    vals, bs = [], []
    for c in range(3):
        v = rng.uniform(-1, 1, len(cl))
        diag = rows == cl
        v[diag] = 0
        rs = np.zeros(n)
        np.add.at(rs, rows, np.abs(v))
        v[diag] = (1.5 + c) * rs[rows[diag]] + 0.1
        vals.append(np.ascontiguousarray(v))
        bs.append(rng.standard_normal(n))
    xs = [np.zeros(n) for _ in range(3)]
    L = _lib.lib()
    dpp = C.POINTER(C.c_double) * 3
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    it = (C.c_int * 3)()
    res = (C.c_double * 3)()
    st = (C.c_int * 3)()
    rc = L.sysu_csr_bicgstab_batched3(n, ip(rp), ip(cl), dpp(*[dp(v) for v in vals]), dpp(*[dp(b) for b in bs]),
                                      dpp(*[dp(x) for x in xs]), 500, 1e-12, it, res, st)
    assert rc == 0, L.sysu_csr_last_error()
    for c in range(3):
        xr, itr, resr, str_ = csr_solve(rp, cl, vals[c], bs[c], method="BiCGSTAB", precond="Jacobi", maxit=500,
                                        eps=1e-12)
        assert st[c] == 0 and str_ == 0 and res[c] < 1e-12
        assert abs(it[c] - itr) <= 1, (c, it[c], itr)
        assert _rel(xs[c], xr) < 1e-10, c


@pytest.mark.parametrize("iters", [200])
def test_scalars_batched_reaches_the_same_steady_state(iters):
    with tempfile.TemporaryDirectory() as d:
        p = mg.write_case(d, mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", iters + 1, turb=True))
        out = {}
        for name, opts in (("sequential", {}), ("batched", {"scalars_batched": 1})):
            o = {"rtc": 1e-12}
            o.update(opts)
            with NavierStokesSolver(p, o) as s:
                s.iterate(iters)
                assert max(s.Residual) < 1e-9, (name, s.Residual)
                out[name] = {f: s.get(f) for f in ("U", "V", "W", "P", "T", "TE", "ED", "VisTur", "solid_T")}
                st = s.solve_stats()
                for eq in ("k", "eps", "T"):
                    assert st[eq]["status"][0] == 0, (eq, st[eq])
    for f, a in out["sequential"].items():
        assert _rel(out["batched"][f], a) < 1e-6, (f, _rel(out["batched"][f], a))

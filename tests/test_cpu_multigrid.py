"""CPU tests of the aggregation multigrid's host side and of its numpy oracle.

The hierarchy the library builds on the host (csrc/amg_setup.cpp, exported as
sysu_mg_hierarchy / sysu_mg_level; no device work) must equal the restatement in
oracle/amg_np.py exactly: the same aggregate of every row at every level, and the
same coarse matrices entry for entry (the Galerkin sums are taken in the same
order, so the values are bit-identical).  The oracle's cycle is checked for the
properties the flexible CG relies on: symmetry, a definite preconditioned
operator, and far fewer iterations than Jacobi-CG.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
from oracle import amg_np  # noqa: E402
from oracle.gnn_np import laplacian_3d
from sysu_cfd_heat_gb300._lib import lib


neumann_3d = amg_np.neumann_3d


def _lib_hierarchy(rp, cl, vl, theta, dense_max):
    L = lib()
    n = len(rp) - 1
    ip = C.POINTER(C.c_int)
    rp_, cl_ = np.ascontiguousarray(rp, np.int32), np.ascontiguousarray(cl, np.int32)
    vl_ = np.ascontiguousarray(vl, np.float64)
    args = (n, rp_.ctypes.data_as(ip), cl_.ctypes.data_as(ip), vl_.ctypes.data_as(C.POINTER(C.c_double)),
            theta, dense_max)
    nlev = C.c_int()
    rows = (C.c_int * 16)()
    nnz = (C.c_long * 16)()
    assert L.sysu_mg_hierarchy(*args, 16, C.byref(nlev), rows, nnz) == 0, L.sysu_mg_last_error()
    out = []
    for l in range(nlev.value):
        m = rows[l]
        agg = np.full(m, -1, np.int32)
        rpo = np.zeros(m + 1, np.int32)
        clo = np.zeros(nnz[l], np.int32)
        vlo = np.zeros(nnz[l])
        assert L.sysu_mg_level(*args, l, agg.ctypes.data_as(ip), rpo.ctypes.data_as(ip), clo.ctypes.data_as(ip),
                               vlo.ctypes.data_as(C.POINTER(C.c_double))) == 0, L.sysu_mg_last_error()
        out.append((m, agg, rpo, clo, vlo))
    return out


@pytest.mark.parametrize("kind,shape,theta", [("dirichlet", (9, 8, 7), 0.25), ("neumann", (10, 9, 8), 0.25),
                                              ("dirichlet", (12, 10, 9), 0.08)])
def test_host_hierarchy_equals_oracle(kind, shape, theta):
    gen = laplacian_3d if kind == "dirichlet" else neumann_3d
    rp, cl, vl = gen(*shape, seed=4) if kind == "neumann" else gen(*shape, seed=4, negative=True)
    dense_max = 40
    ours = _lib_hierarchy(rp, cl, vl, theta, dense_max)
    ref = amg_np.hierarchy(rp, cl, vl, theta=theta, dense_max=dense_max)
    assert len(ours) == len(ref) >= 3
    for l, ((m, agg, rpo, clo, vlo), R) in enumerate(zip(ours, ref)):
        assert m == R.n
        if R.agg is not None:
            np.testing.assert_array_equal(agg, R.agg)
        np.testing.assert_array_equal(rpo, R.rp)
        np.testing.assert_array_equal(clo, R.col)
        np.testing.assert_array_equal(vlo, R.val)  # same summation order: bit-identical
    assert ref[-1].n <= dense_max


def test_oracle_cycle_is_symmetric_definite_and_fast():
    rp, cl, vl = neumann_3d(14, 12, 10, seed=5)
    lv = amg_np.hierarchy(rp, cl, vl, dense_max=60)
    n = lv[0].n
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    x -= x.mean()
    y -= y.mean()
    Mx, My = amg_np.vcycle(lv, x), amg_np.vcycle(lv, y)
    assert abs(y @ Mx - x @ My) <= 1e-10 * abs(y @ Mx)
    # negative definite operator -> M negative definite on the consistent space
    assert x @ Mx < 0 and y @ My < 0
    b = rng.standard_normal(n)
    b -= b.mean()  # consistent right-hand side of the singular system
    xm, itm, resm = amg_np.fcg(lv, b, lambda r: amg_np.vcycle(lv, r), eps=1e-8, maxit=500)
    xj, itj, resj = amg_np.fcg(lv, b, lambda r: r / lv[0].diag, eps=1e-8, maxit=5000)
    assert resm < 1e-8 and resj < 1e-8
    assert itm * 4 < itj, (itm, itj)
    d = (xm - xm.mean()) - (xj - xj.mean())
    assert np.linalg.norm(d) <= 1e-6 * np.linalg.norm(xj - xj.mean())


def test_cycle_fixed_plus_jacobi_is_the_vcycle():
    rp, cl, vl = laplacian_3d(8, 7, 6, seed=2, negative=True)
    lv = amg_np.hierarchy(rp, cl, vl, dense_max=30)
    r = np.random.default_rng(3).standard_normal(lv[0].n)
    z2, t = amg_np.cycle_fixed(lv, r)
    np.testing.assert_allclose(t, r - lv[0].matvec(z2), rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(z2 + 0.8 / lv[0].diag * t, amg_np.vcycle(lv, r), rtol=1e-14, atol=1e-14)

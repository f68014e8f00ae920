"""Momentum form of the mixed BiCGSTAB (sysu_csr_bicgstab3, mixed=1): u, v, w of one
matrix with FP32 recurrences on interleaved vectors, x accumulated in FP64 and the
FP64 residual replacing the FP32 one.  It stops on the FP64 form's test
||b - A x|| / ||b|| < eps made on the true residual, so per component the solution
agrees with the FP64 batched solve (mixed=0) to the conditioning times eps, and the
reported residual is the true one."""
import os

import numpy as np
import pytest

from sysu_cfd_heat_gb300.solver import SysuError, csr_bicgstab3, csr_spmv

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _convection_diffusion(nx, ny, nz, peclet, seed):
    """Upwind convection-diffusion on a box grid: non-symmetric, an M-matrix, with
    three right-hand sides of different scales."""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    idx = np.arange(n).reshape(nz, ny, nx)
    rows, cols, vals = [], [], []
    for axis, vel in ((2, 1.0), (1, 0.5), (0, -0.3)):
        lo = np.take(idx, range(0, idx.shape[axis] - 1), axis=axis).ravel()
        hi = np.take(idx, range(1, idx.shape[axis]), axis=axis).ravel()
        w = 1.0 + 0.2 * rng.random(lo.size)
        c = peclet * vel
        rows += [lo, hi]
        cols += [hi, lo]
        vals += [-(w + max(-c, 0.0)), -(w + max(c, 0.0))]
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    diag = np.zeros(n)
    np.add.at(diag, rows, -vals)
    diag += 0.05
    rows = np.concatenate([rows, np.arange(n)])
    cols = np.concatenate([cols, np.arange(n)])
    vals = np.concatenate([vals, diag])
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, rows + 1, 1)
    B = np.stack([rng.standard_normal(n), 1e-6 * rng.standard_normal(n), 1e3 * rng.random(n)])
    return np.cumsum(rp).astype(np.int32), cols.astype(np.int32), vals, B


def _true_res(rp, cl, vl, x, b):
    return np.linalg.norm(b - csr_spmv(rp, cl, vl, x)) / np.linalg.norm(b)


@pytest.mark.parametrize("peclet", [0.5, 4.0])
@pytest.mark.parametrize("eps", [1e-8, 1e-12])
def test_mixed3_matches_fp64_batched(peclet, eps):
    rp, cl, vl, B = _convection_diffusion(24, 20, 16, peclet, seed=3)
    X64, it64, _, st64, _ = csr_bicgstab3(rp, cl, vl, B, mixed=False, maxit=5000, eps=eps)
    Xm, itm, resm, stm, ref = csr_bicgstab3(rp, cl, vl, B, mixed=True, maxit=5000, eps=eps)
    assert st64 == [0, 0, 0] and stm == [0, 0, 0], (st64, stm)
    assert ref >= 3  # at least one replacement per component
    for c in range(3):
        true = _true_res(rp, cl, vl, Xm[c], B[c])
        assert true < eps and abs(true - resm[c]) <= 1e-3 * resm[c] + 1e-18, (c, true, resm[c])
        assert _rel(Xm[c], X64[c]) < 1e3 * eps, c
        assert itm[c] <= 3 * it64[c] + 10, (itm, it64)


def test_mixed3_is_deterministic():
    rp, cl, vl, B = _convection_diffusion(20, 18, 14, 2.0, seed=7)
    a = csr_bicgstab3(rp, cl, vl, B, mixed=True, eps=1e-10, maxit=3000)
    b = csr_bicgstab3(rp, cl, vl, B, mixed=True, eps=1e-10, maxit=3000)
    assert np.array_equal(a[0], b[0]) and a[1] == b[1] and a[4] == b[4]


def test_mixed3_on_reference_momentum_systems():
    """u, v, w of the reference's first outer iteration (one matrix; w has a zero
    right-hand side), solved as the reference did to 1e-13 with Jacobi(1.2)."""
    g = np.load(os.path.join(GOLD, "cavity_hex6_tight.npz"))
    rp, cl, vl = g["solve0_rowptr"], g["solve0_col"], g["solve0_val"]
    for k in (1, 2):
        assert np.array_equal(g[f"solve{k}_val"], vl)
    B = np.stack([g[f"solve{k}_b"] for k in range(3)])
    X, it, res, st, _ = csr_bicgstab3(rp, cl, vl, B, mixed=True, maxit=2000, eps=1e-13, omega=1.2)
    assert st == [0, 0, 0], st
    assert it[2] == 0 and not X[2].any()  # zero right-hand side from x0 = 0: no iteration
    for k in (0, 1):
        assert res[k] < 1e-13
        assert _rel(X[k], g[f"solve{k}_x"]) < 1e-9, k


def test_mixed3_edge_cases():
    rp, cl, vl, B = _convection_diffusion(12, 10, 8, 1.0, seed=5)
    n = len(rp) - 1
    # a converged start (x0 = the FP64 solution) and a zero right-hand side take no
    # iteration; the third component solves as usual
    X64, _, _, _, _ = csr_bicgstab3(rp, cl, vl, B, eps=1e-12, maxit=3000)
    B2 = B.copy()
    B2[1] = 0.0
    X0 = np.stack([X64[0], np.zeros(n), np.zeros(n)])
    X, it, res, st, _ = csr_bicgstab3(rp, cl, vl, B2, X0, mixed=True, eps=1e-10, maxit=3000)
    assert st == [0, 0, 0] and it[0] == 0 and it[1] == 0 and it[2] > 0, (st, it)
    assert np.array_equal(X[0], X64[0]) and not X[1].any()
    assert _true_res(rp, cl, vl, X[2], B2[2]) < 1e-10
    # the iteration cap: status 1 (max iterations) with the cap's count
    X, it, res, st, _ = csr_bicgstab3(rp, cl, vl, B, mixed=True, eps=1e-14, maxit=3)
    assert st == [1, 1, 1] and it == [3, 3, 3], (st, it)
    for c in range(3):
        assert abs(_true_res(rp, cl, vl, X[c], B[c]) - res[c]) <= 1e-6 * res[c]
    # maxit 0: nothing runs
    X, it, res, st, _ = csr_bicgstab3(rp, cl, vl, B, mixed=True, eps=1e-8, maxit=0)
    assert st == [1, 1, 1] and it == [0, 0, 0] and not X.any()


def test_mixed3_unreachable_tolerance_ends():
    """eps below what FP64 can reach: the replacements stop lowering the residual,
    the component is handed to the FP64 solve from its x, and the call returns
    with the residual at FP64 round-off."""
    rp, cl, vl, B = _convection_diffusion(12, 10, 8, 1.0, seed=9)
    X, it, res, st, _ = csr_bicgstab3(rp, cl, vl, B, mixed=True, eps=1e-19, maxit=400)
    for c in range(3):
        assert _true_res(rp, cl, vl, X[c], B[c]) < 1e-13, c
        assert it[c] > 0


def test_mixed3_argument_errors():
    rp, cl, vl, B = _convection_diffusion(6, 5, 4, 1.0, seed=1)
    with pytest.raises(SysuError):
        csr_bicgstab3(rp, cl, vl, B, mixed=True, inner_tol=0.0)
    with pytest.raises(SysuError):
        csr_bicgstab3(rp, cl, vl, B, mixed=True, inner_tol=1.0)
    with pytest.raises(SysuError):
        csr_bicgstab3(rp, cl, vl, B, mixed=True, eps=0.0)

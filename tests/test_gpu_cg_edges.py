"""Edge cases of the GPU CG kernels (FP64 and FP32 with reliable updates) against the
oracle's Jacobi-PCG (oracle/simple_np.py, Templates Fig. 2.5, the recurrences of
LASPack's CGIter).

The kernels stream tiles of 32 slices (1024 rows) through a ring of shared-memory
slots; the sizes below cover: fewer rows than a warp, ragged last slices (n not a
multiple of 32 or 4), CTAs owning a single tile (ring depth 1), many tiles per CTA,
rows wide enough to shrink the tile (SELL width 31) and rows too wide for any slot
(the matrix is then read from global memory).
"""
import numpy as np
import pytest

from oracle.simple_np import cg as oracle_cg
from sysu_cfd_heat_gb300.solver import csr_solve, csr_spmv

pytestmark = pytest.mark.gpu


def spd_csr(n, extra, seed, wide_row=False):
    """Symmetric, strictly diagonally dominant matrix: a chain plus `extra` random
    symmetric couplings per row; optionally row/column 0 coupled to every row."""
    rng = np.random.default_rng(seed)
    ent = {}

    def add(i, j, v):
        ent[(i, j)] = ent.get((i, j), 0.0) + v
        ent[(j, i)] = ent.get((j, i), 0.0) + v

    for i in range(n - 1):
        add(i, i + 1, -rng.uniform(0.5, 1.5))
    for i in range(n):
        for _ in range(extra):
            j = int(rng.integers(0, n))
            if j != i:
                add(i, j, -rng.uniform(0.1, 1.0))
    if wide_row:
        for j in range(1, n):
            add(0, j, -rng.uniform(0.01, 0.1))
    rows = [[] for _ in range(n)]
    off = np.zeros(n)
    for (i, j), v in ent.items():
        rows[i].append((j, v))
        off[i] += abs(v)
    rp, cl, vl = [0], [], []
    for i in range(n):
        rows[i].append((i, off[i] * rng.uniform(1.05, 1.5) + 1e-3))
        rows[i].sort()
        for j, v in rows[i]:
            cl.append(j)
            vl.append(v)
        rp.append(len(cl))
    return np.array(rp, np.int32), np.array(cl, np.int32), np.array(vl)


def oracle(rp, cl, vl, b, maxit, eps, omega):
    n = len(rp) - 1
    d = np.zeros(n)
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            if cl[k] == i:
                d[i] += vl[k]
    return oracle_cg((rp, cl, vl, d), b, np.zeros(n), maxit, eps, omega)


CASES = [
    # n, extra couplings per row, wide row
    (1, 0, False),
    (2, 0, False),
    (5, 1, False),
    (31, 2, False),
    (33, 2, False),
    (1023, 2, False),
    (1025, 3, False),
    (4099, 2, False),
    (40001, 2, False),
    (3000, 9, False),   # SELL width 31: smaller tiles
    (700, 1, True),     # one 700-entry row: matrix read from global memory
]


@pytest.mark.parametrize("n,extra,wide", CASES)
def test_cg_fp64_matches_oracle(n, extra, wide):
    rp, cl, vl = spd_csr(n, extra, seed=n + extra, wide_row=wide)
    b = np.random.default_rng(7).standard_normal(n)
    eps, omega = 1e-10, 1.2
    xo, ito, reso = oracle(rp, cl, vl, b, 5000, eps, omega)
    x, it, res, st = csr_solve(rp, cl, vl, b, None, method="CG", maxit=5000, eps=eps, omega=omega)
    assert st == 0 and res < eps
    assert abs(it - ito) <= max(1, ito // 50), (it, ito)
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo) + 1e-300
    r = b - csr_spmv(rp, cl, vl, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2 * eps


@pytest.mark.parametrize("n,extra,wide", CASES)
def test_cg_mixed_reaches_fp64_tolerance(n, extra, wide):
    rp, cl, vl = spd_csr(n, extra, seed=n + extra, wide_row=wide)
    b = np.random.default_rng(8).standard_normal(n)
    eps, omega = 1e-10, 1.2
    xo, ito, reso = oracle(rp, cl, vl, b, 5000, eps, omega)
    x, it, res, st = csr_solve(rp, cl, vl, b, None, method="CG-mixed", maxit=20000, eps=eps, omega=omega)
    assert st == 0 and res < eps
    # the reported residual is the true FP64 one
    r = b - csr_spmv(rp, cl, vl, x)
    assert abs(np.linalg.norm(r) / np.linalg.norm(b) - res) <= 1e-3 * res + 1e-16
    assert np.linalg.norm(x - xo) <= 1e-7 * np.linalg.norm(xo) + 1e-300


def test_cg_iteration_cap_and_zero_rhs():
    rp, cl, vl = spd_csr(2000, 2, seed=3)
    b = np.random.default_rng(9).standard_normal(2000)
    x, it, res, st = csr_solve(rp, cl, vl, b, None, method="CG", maxit=3, eps=1e-14, omega=1.0)
    xo, ito, reso = oracle(rp, cl, vl, b, 3, 1e-14, 1.0)
    assert st == 1 and it == 3 == ito
    assert abs(res - reso) <= 1e-9 * reso
    assert np.linalg.norm(x - xo) <= 1e-11 * np.linalg.norm(xo)
    x, it, res, st = csr_solve(rp, cl, vl, np.zeros(2000), None, method="CG", maxit=10, eps=1e-8)
    assert st == 0 and it == 0 and not np.any(x)
    x, it, res, st = csr_solve(rp, cl, vl, np.zeros(2000), None, method="CG-mixed", maxit=10, eps=1e-8)
    assert st == 0 and it == 0 and not np.any(x)


def grid5(nx, ny, seed, dominance=1.5):
    """5-point stencil on an nx x ny grid, random symmetric positive couplings."""
    rng = np.random.default_rng(seed)
    n = nx * ny
    idx = np.arange(n).reshape(ny, nx)
    wx = rng.uniform(0.5, 1.5, (ny, nx - 1))
    wy = rng.uniform(0.5, 1.5, (ny - 1, nx))
    I = np.concatenate([idx[:, :-1].ravel(), idx[:, 1:].ravel(), idx[:-1, :].ravel(), idx[1:, :].ravel()])
    J = np.concatenate([idx[:, 1:].ravel(), idx[:, :-1].ravel(), idx[1:, :].ravel(), idx[:-1, :].ravel()])
    V = -np.concatenate([wx.ravel(), wx.ravel(), wy.ravel(), wy.ravel()])
    diag = np.zeros(n)
    np.add.at(diag, I, -V)
    I = np.concatenate([I, np.arange(n)])
    J = np.concatenate([J, np.arange(n)])
    V = np.concatenate([V, dominance * diag])
    o = np.lexsort((J, I))
    I, J, V = I[o], J[o], V[o]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, I + 1, 1)
    return np.cumsum(rp).astype(np.int32), J.astype(np.int32), V


@pytest.mark.parametrize("method", ["CG", "CG-mixed"])
def test_cg_many_tiles_per_cta(method):
    """1M rows: every CTA streams several tiles per phase through a full ring."""
    rp, cl, vl = grid5(1000, 1000, seed=11)
    b = np.random.default_rng(12).standard_normal(len(rp) - 1)
    eps, omega = 1e-9, 1.0
    xo, ito, reso = oracle(rp, cl, vl, b, 2000, eps, omega)
    x, it, res, st = csr_solve(rp, cl, vl, b, None, method=method, maxit=2000, eps=eps, omega=omega)
    assert st == 0 and res < eps
    if method == "CG":
        assert abs(it - ito) <= 1, (it, ito)
    r = b - csr_spmv(rp, cl, vl, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2 * eps
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)


def grid7(m, seed, dominance):
    """7-point stencil on an m^3 grid, random symmetric positive couplings, diagonal
    `dominance` times the row's coupling sum (rows of up to 7 entries)."""
    rng = np.random.default_rng(seed)
    n = m ** 3
    idx = np.arange(n).reshape(m, m, m)
    Is, Js, Vs = [], [], []
    for ax in range(3):
        a = np.take(idx, range(m - 1), axis=ax).ravel()
        b = np.take(idx, range(1, m), axis=ax).ravel()
        w = -rng.uniform(0.5, 1.5, a.size)
        Is += [a, b]
        Js += [b, a]
        Vs += [w, w]
    I, J, V = np.concatenate(Is), np.concatenate(Js), np.concatenate(Vs)
    diag = np.zeros(n)
    np.add.at(diag, I, -V)
    I = np.concatenate([I, np.arange(n)])
    J = np.concatenate([J, np.arange(n)])
    V = np.concatenate([V, dominance * diag])
    o = np.lexsort((J, I))
    I, J, V = I[o], J[o], V[o]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, I + 1, 1)
    return np.cumsum(rp).astype(np.int32), J.astype(np.int32), V


def test_cg_wide_rows_above_one_million():
    """128^3 = 2,097,152 rows of up to 7 entries: the FP64 kernel's one-tile-at-a-time
    form on 1024 threads (rows wider than 5 at >= 2^20 rows; the hex-mesh p' systems
    of the large channel run it), and the FP32 form on the same system."""
    rp, cl, vl = grid7(128, seed=21, dominance=1.01)
    n = len(rp) - 1
    assert np.diff(rp).max() == 7 and n >= 1 << 20
    b = np.random.default_rng(22).standard_normal(n)
    eps = 1e-9
    d = vl[cl == np.repeat(np.arange(n), np.diff(rp))]
    xo, ito, reso = oracle_cg((rp, cl, vl, d), b, np.zeros(n), 5000, eps, 1.0)
    assert reso < eps
    for method in ("CG", "CG-mixed"):
        x, it, res, st = csr_solve(rp, cl, vl, b, None, method=method, maxit=5000, eps=eps, omega=1.0)
        assert st == 0 and res < eps, (method, st, it, res)
        if method == "CG":
            assert abs(it - ito) <= 1, (it, ito)
        r = b - csr_spmv(rp, cl, vl, x)
        assert np.linalg.norm(r) / np.linalg.norm(b) < 2 * eps, method
        assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo), method

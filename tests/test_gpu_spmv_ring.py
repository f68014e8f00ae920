"""The standalone SpMV forms give the same y bit for bit.

The persistent ring product (matrix tiles streamed through shared memory by bulk
copies, x gathered one tile ahead) and the per-warp cp.async pipeline against the
one-row-per-thread kernel and a numpy CSR product, on ragged sizes, rows wider
than the gathers held in registers or the staged width, and rows too wide for a
ring slot (read from global memory).
"""
import numpy as np
import pytest

from sysu_cfd_heat_gb300.solver import csr_spmv, set_spmv_variant

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _default_variant():
    yield
    set_spmv_variant(0)


def _random_csr(n, wmin, wmax, seed, wide_rows=()):
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for i in range(n):
        w = int(rng.integers(wmin, wmax + 1)) if i not in wide_rows else min(n, 300)
        nb = rng.choice(n, size=min(n, w), replace=False)
        nb = [i] + [int(c) for c in nb if c != i][: max(0, w - 1)]
        rows.append(len(nb))
        cols.extend(nb)
        vals.extend(rng.standard_normal(len(nb)).tolist())
    rowptr = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    return rowptr, np.array(cols, np.int32), np.array(vals, np.float64)


def _numpy_spmv(rowptr, col, val, x):
    y = np.zeros(len(rowptr) - 1)
    for i in range(len(y)):
        a, b = rowptr[i], rowptr[i + 1]
        y[i] = np.dot(val[a:b], x[col[a:b]])
    return y


@pytest.mark.parametrize("n,wmin,wmax,wide", [
    (40003, 1, 9, ()),          # ragged slices, widths past the register gathers
    (20000, 5, 5, ()),          # tet-like, uniform width
    (31, 1, 4, ()),             # one partial slice
    (5000, 2, 7, (17, 4321)),   # two rows of 300 entries: read from global memory by both forms
    (3000, 7, 12, ()),          # slices wider than the staged width of the cp.async form
])
def test_ring_matches_stream(n, wmin, wmax, wide):
    rowptr, col, val = _random_csr(n, wmin, wmax, seed=n + wmax, wide_rows=wide)
    x = np.random.default_rng(7).standard_normal(n)
    set_spmv_variant(0)
    y0 = csr_spmv(rowptr, col, val, x)
    set_spmv_variant(100)
    y1 = csr_spmv(rowptr, col, val, x)
    assert np.array_equal(y0, y1)
    set_spmv_variant(200)
    y2 = csr_spmv(rowptr, col, val, x)
    assert np.array_equal(y0, y2)
    set_spmv_variant(300)
    y3 = csr_spmv(rowptr, col, val, x)
    set_spmv_variant(0)
    assert np.array_equal(y0, y3)
    if n <= 20000:
        ref = _numpy_spmv(rowptr, col, val, x)
        np.testing.assert_allclose(y1, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("variant", [100, 200, 300])
def test_single_row_and_empty(variant):
    set_spmv_variant(variant)
    y = csr_spmv(np.array([0, 1], np.int32), np.array([0], np.int32), np.array([2.5]), np.array([4.0]))
    assert y.tolist() == [10.0]
    y = csr_spmv(np.array([0], np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0))
    assert y.size == 0


def test_bad_variant_rejected():
    with pytest.raises(RuntimeError):
        set_spmv_variant(7)


@pytest.mark.parametrize("variant", [0, 300])
def test_steady_state_timing_of_an_assembled_matrix(variant):
    """sysu_solver_spmv_timing_steady (products back to back, alternating between
    the operands and a full copy of them) runs on an assembled matrix and gives a
    per-product time in the range of the flushed single-product timing."""
    import tempfile

    from sysu_cfd_heat_gb300 import meshgen as mg
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_tet(20, 18, 16, jitter=0.2), mg.cavity_param("x", 5, mu=0.01))
        with NavierStokesSolver(p, {"rtc": 1e-8, "spmv_variant": variant}) as s:
            s.iterate(1)
            for which in ("p", "mom"):
                for fp32 in (False, True):
                    steady = s.spmv_timing(which, fp32, 4, steady=True)
                    flushed = s.spmv_timing(which, fp32, 4)
                    assert 0.0 < steady < 10.0 * flushed + 1.0, (which, fp32, steady, flushed)

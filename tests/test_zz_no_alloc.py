"""GPU test of sysu_csr_cg_noalloc, the Jacobi-CG entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (applications that own all device
memory through their own pool, loops that must not pay cudaMalloc's device-wide
synchronisation): they pass their own device buffers and the solver's scratch is a
static device array.  This test plays such a caller -- the buffers come from torch --
and checks two calls in a row against sysu_csr_solve (CG, Jacobi) on the same systems.
The file sorts last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from sysu_cfd_heat_gb300._lib import LIB_PATH
from sysu_cfd_heat_gb300.solver import csr_solve

pytestmark = pytest.mark.gpu

MAX_ROWS = 262144  # SYSU_NOALLOC_MAX_ROWS


def poisson_csr(m, shift):
    """7-point 3-D Laplacian on m^3 nodes plus shift*I (SPD), 0-based CSR."""
    n = m ** 3
    idx = np.arange(n).reshape(m, m, m)
    rows, cols, vals = [idx.ravel()], [idx.ravel()], [np.full(n, 6.0 + shift)]
    for ax in range(3):
        for d in (-1, 1):
            src = np.take(idx, range(max(0, -d), m - max(0, d)), axis=ax).ravel()
            dst = np.take(idx, range(max(0, d), m - max(0, -d)), axis=ax).ravel()
            rows.append(src); cols.append(dst); vals.append(np.full(src.size, -1.0))
    r, c, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    rowptr = np.zeros(n + 1, np.int32)
    np.add.at(rowptr, r + 1, 1)
    return np.cumsum(rowptr).astype(np.int32), c.astype(np.int32), v


def _fn():
    lib = C.CDLL(LIB_PATH)
    f = lib.sysu_csr_cg_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                  C.c_double, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int)]
    lib.sysu_noalloc_last_error.restype = C.c_char_p
    return f, lib


def test_noalloc_cg_matches_csr_solve_on_two_calls():
    torch = pytest.importorskip("torch")
    f, _ = _fn()
    rp, cl, vl = poisson_csr(48, 0.02)  # 110,592 rows
    n = len(rp) - 1
    d_rp = torch.from_numpy(rp).cuda()
    d_cl = torch.from_numpy(cl).cuda()
    d_vl = torch.from_numpy(vl).cuda()
    rng = np.random.default_rng(7)
    for call in range(2):  # two calls in a row share the static scratch
        b = rng.standard_normal(n)
        x_ref, it_ref, res_ref, st_ref = csr_solve(rp, cl, vl, b, None, method="CG", precond="Jacobi", maxit=2000,
                                                   eps=1e-10, omega=1.0)
        assert st_ref == 0
        d_b = torch.from_numpy(b).cuda()
        d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        it, res, st = C.c_int(), C.c_double(), C.c_int()
        rc = f(n, d_rp.data_ptr(), d_cl.data_ptr(), d_vl.data_ptr(), d_b.data_ptr(), d_x.data_ptr(), 2000, 1e-10,
               1.0, None, C.byref(it), C.byref(res), C.byref(st))
        assert rc == 0
        assert st.value == 0, (st.value, it.value, res.value)
        assert res.value < 1e-10
        assert abs(it.value - it_ref) <= 2, (it.value, it_ref)
        x = d_x.cpu().numpy()
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9


def _call(f, n, d_rp, d_cl, d_vl, d_b, d_x, maxit, eps, stream=None):
    it, res, st = C.c_int(), C.c_double(), C.c_int()
    rc = f(n, d_rp.data_ptr(), d_cl.data_ptr(), d_vl.data_ptr(), d_b.data_ptr(), d_x.data_ptr(), maxit, eps, 1.0,
           stream, C.byref(it), C.byref(res), C.byref(st))
    return rc, it.value, res.value, st.value


def test_noalloc_cg_on_a_stream_from_a_nonzero_start_at_the_size_limit():
    """n = 64^3 = SYSU_NOALLOC_MAX_ROWS (the partial sums and D^-1 sit at the end of the
    array), x0 random (the b - A x0 pass runs before any write of x), on a torch
    stream rather than the default one; then a 5-iteration cap ends with status 1."""
    torch = pytest.importorskip("torch")
    f, _ = _fn()
    rp, cl, vl = poisson_csr(64, 0.05)
    n = len(rp) - 1
    assert n == MAX_ROWS
    rng = np.random.default_rng(11)
    b = rng.standard_normal(n)
    x0 = rng.standard_normal(n)
    x_ref, it_ref, _, st_ref = csr_solve(rp, cl, vl, b, x0.copy(), method="CG", precond="Jacobi", maxit=3000,
                                         eps=1e-10, omega=1.0)
    assert st_ref == 0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        d_rp, d_cl, d_vl = (torch.from_numpy(a).cuda() for a in (rp, cl, vl))
        d_b, d_x = torch.from_numpy(b).cuda(), torch.from_numpy(x0).cuda()
    s.synchronize()
    for call in range(2):
        d_x.copy_(torch.from_numpy(x0).cuda())
        torch.cuda.synchronize()
        rc, it, res, st = _call(f, n, d_rp, d_cl, d_vl, d_b, d_x, 3000, 1e-10, C.c_void_p(s.cuda_stream))
        assert rc == 0 and st == 0, (rc, st, it, res)
        assert abs(it - it_ref) <= 2, (it, it_ref)
        s.synchronize()
        x = d_x.cpu().numpy()
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9
    d_x.copy_(torch.from_numpy(x0).cuda())
    torch.cuda.synchronize()
    rc, it, res, st = _call(f, n, d_rp, d_cl, d_vl, d_b, d_x, 5, 1e-10, C.c_void_p(s.cuda_stream))
    x5, it5, res5, st5 = csr_solve(rp, cl, vl, b, x0.copy(), method="CG", precond="Jacobi", maxit=5, eps=1e-10,
                                   omega=1.0)
    assert rc == 0 and st == 1 and it == 5 and st5 == 1, (rc, st, it, st5)
    assert abs(res - res5) <= 1e-9 * res5, (res, res5)
    s.synchronize()
    assert np.linalg.norm(d_x.cpu().numpy() - x5) / np.linalg.norm(x5) < 1e-12


def test_noalloc_reports_a_malformed_matrix_without_solving():
    """A column index outside 0..n-1 and a row with no diagonal are input errors
    naming the lowest such row; x is left untouched."""
    torch = pytest.importorskip("torch")
    f, lib = _fn()
    rp, cl, vl = poisson_csr(16, 0.1)
    n = len(rp) - 1
    b = np.ones(n)
    for row, kind in ((37, "col"), (5, "diag")):
        c, v = cl.copy(), vl.copy()
        if kind == "col":
            c[rp[row] + 1] = n + 3
        else:
            v[(c == row) & (np.arange(len(c)) >= rp[row]) & (np.arange(len(c)) < rp[row + 1])] = 0.0
        d_rp, d_cl, d_vl = (torch.from_numpy(a).cuda() for a in (rp, c, v))
        d_b = torch.from_numpy(b).cuda()
        d_x = torch.full((n,), 0.5, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc, _, _, _ = _call(f, n, d_rp, d_cl, d_vl, d_b, d_x, 100, 1e-8)
        assert rc == 1, rc
        msg = lib.sysu_noalloc_last_error().decode()
        assert f"row {row} " in msg, msg
        assert bool(torch.all(d_x == 0.5))
    # a well-formed call afterwards is unaffected by the stored check result
    d_rp, d_cl, d_vl = (torch.from_numpy(a).cuda() for a in (rp, cl, vl))
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc, it, res, st = _call(f, n, d_rp, d_cl, d_vl, torch.from_numpy(b).cuda(), d_x, 1000, 1e-10)
    assert rc == 0 and st == 0 and res < 1e-10


def test_noalloc_refuses_a_capturing_stream():
    """The call reads its result back, so it cannot sit inside a CUDA graph: on a
    stream under capture it returns an input error and queues nothing."""
    torch = pytest.importorskip("torch")
    f, lib = _fn()
    rp, cl, vl = poisson_csr(8, 0.1)
    n = len(rp) - 1
    d_rp, d_cl, d_vl = (torch.from_numpy(a).cuda() for a in (rp, cl, vl))
    d_b = torch.ones(n, dtype=torch.float64, device="cuda")
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    out = {}
    with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
        d_x.add_(0.0)
        out["r"] = _call(f, n, d_rp, d_cl, d_vl, d_b, d_x, 100, 1e-8,
                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert out["r"][0] == 1, out
    assert b"captured" in lib.sysu_noalloc_last_error()


def test_noalloc_rejects_systems_beyond_its_scratch():
    f, lib = _fn()
    it, res, st = C.c_int(), C.c_double(), C.c_int()
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = f(MAX_ROWS + 1, dummy, dummy, dummy, dummy, dummy, 10, 1e-8, 1.0, None, C.byref(it), C.byref(res),
           C.byref(st))
    assert rc == 1
    assert b"262144" in lib.sysu_noalloc_last_error()

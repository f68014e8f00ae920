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


def test_noalloc_rejects_systems_beyond_its_scratch():
    f, lib = _fn()
    it, res, st = C.c_int(), C.c_double(), C.c_int()
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = f(MAX_ROWS + 1, dummy, dummy, dummy, dummy, dummy, 10, 1e-8, 1.0, None, C.byref(it), C.byref(res),
           C.byref(st))
    assert rc == 1
    assert b"262144" in lib.sysu_noalloc_last_error()

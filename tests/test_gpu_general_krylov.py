"""GPU GMRES(m), PCG with SSOR / ILU(0), and the reference's own solver mode.

The same LASPack calls run against the GPU library (libsysucfd.so) and the oracle's
CPU LASPack restatement (oracle/_ref/liblaspack_cpu.so): GMRES(10) right
preconditioned, SSOR(omega) and ILU(0) in natural row order, CG.  The GPU sweeps are
level-scheduled but perform the same operations per row, and GMRES orthogonalises by
classical Gram-Schmidt applied twice instead of modified Gram-Schmidt, so iteration
counts agree within one and solutions within the tolerance.  At the SIMPLE level,
option "reference_solvers" (GMRES + SSOR and CG + SSOR as the reference calls them)
reaches the reference's fields on the tight-tolerance fixtures.
"""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import make_golden
from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300._lib import LIB_PATH
from sysu_cfd_heat_gb300.solver import NavierStokesSolver, csr_solve

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LAS_CPU = os.path.join(ROOT, "oracle", "_ref", "liblaspack_cpu.so")
GOLD = os.path.join(os.path.dirname(__file__), "golden")


class Vec(C.Structure):
    _fields_ = [("Name", C.c_char_p), ("Dim", C.c_size_t), ("Instance", C.c_int), ("OwnData", C.c_int),
                ("Cmp", C.POINTER(C.c_double))]


class QMat(C.Structure):
    _fields_ = [("Name", C.c_char_p), ("Dim", C.c_size_t), ("Symmetry", C.c_int), ("ElOrder", C.c_int),
                ("Instance", C.c_int), ("OwnData", C.c_int), ("Len", C.c_void_p), ("El", C.c_void_p),
                ("Priv", C.c_void_p)]


def _bind(path):
    L = C.CDLL(path)
    L.Q_Constr.argtypes = [C.POINTER(QMat), C.c_char_p, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int]
    L.Q_SetLen.argtypes = [C.POINTER(QMat), C.c_size_t, C.c_size_t]
    L.Q_SetEntry.argtypes = [C.POINTER(QMat), C.c_size_t, C.c_size_t, C.c_size_t, C.c_double]
    L.Q_Destr.argtypes = [C.POINTER(QMat)]
    L.V_Constr.argtypes = [C.POINTER(Vec), C.c_char_p, C.c_size_t, C.c_int, C.c_int]
    L.SetRTCAccuracy.argtypes = [C.c_double]
    L.SetGMRESRestart.argtypes = [C.c_int]
    L.GetLastAccuracy.restype = C.c_double
    for it in ("CGIter", "BiCGSTABIter", "GMRESIter"):
        getattr(L, it).argtypes = [C.POINTER(QMat), C.POINTER(Vec), C.POINTER(Vec), C.c_int, C.c_void_p, C.c_double]
        getattr(L, it).restype = C.POINTER(Vec)
    for pc in ("JacobiPrecond", "SSORPrecond", "ILUPrecond"):
        getattr(L, pc).argtypes = [C.POINTER(QMat), C.POINTER(Vec), C.POINTER(Vec), C.c_double]
        getattr(L, pc).restype = C.POINTER(Vec)
    return L


@pytest.fixture(scope="module")
def libs():
    if not os.path.exists(LAS_CPU):
        pytest.skip("oracle/_ref/liblaspack_cpu.so not built")
    return _bind(LIB_PATH), _bind(LAS_CPU)


def fv_like(m, nonsym, seed):
    """7-point operator on an m^3 grid with random positive couplings, diagonally
    dominant; nonsym adds an upwind-like convection part."""
    rng = np.random.default_rng(seed)
    n = m ** 3
    A = np.zeros((n, n))
    for i in range(m):
        for j in range(m):
            for k in range(m):
                r = (i * m + j) * m + k
                for d in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
                    a, b, c = i + d[0], j + d[1], k + d[2]
                    if a < m and b < m and c < m:
                        q = (a * m + b) * m + c
                        w = rng.uniform(0.5, 1.5)
                        A[r, q] -= w
                        A[q, r] -= w
                        if nonsym:
                            A[q, r] -= rng.uniform(0.0, 0.8)
    A[np.diag_indices(n)] = -A.sum(axis=1) + 0.05
    return A


def _load(L, A, symmetric):
    n = A.shape[0]
    q = QMat()
    L.Q_Constr(C.byref(q), b"A", n, 1 if symmetric else 0, 0, 0, 1)
    for i in range(n):
        cols = [j for j in range(n) if A[i, j] != 0 and j != i and (not symmetric or j > i)]
        L.Q_SetLen(C.byref(q), i + 1, len(cols) + 1)
        L.Q_SetEntry(C.byref(q), i + 1, 0, i + 1, float(A[i, i]))
        for k, j in enumerate(cols):
            L.Q_SetEntry(C.byref(q), i + 1, k + 1, j + 1, float(A[i, j]))
    return q


def _vec(L, v):
    x = Vec()
    L.V_Constr(C.byref(x), b"v", len(v), 0, 1)
    for i, a in enumerate(v):
        x.Cmp[i + 1] = a
    return x


def _solve(L, it, pc, A, b, sym, eps, omega):
    n = len(b)
    q = _load(L, A, sym)
    x, bb = _vec(L, np.zeros(n)), _vec(L, b)
    L.SetRTCAccuracy(eps)
    L.SetGMRESRestart(10)
    getattr(L, it)(C.byref(q), C.byref(x), C.byref(bb), 2000, C.cast(getattr(L, pc), C.c_void_p), omega)
    out = np.array([x.Cmp[i + 1] for i in range(n)]), L.GetLastNoIter(), L.GetLastAccuracy()
    L.Q_Destr(C.byref(q))
    return out


@pytest.mark.parametrize("it,pc,sym", [
    ("GMRESIter", "SSORPrecond", False), ("GMRESIter", "ILUPrecond", False), ("GMRESIter", "JacobiPrecond", False),
    ("CGIter", "SSORPrecond", True), ("CGIter", "ILUPrecond", True),
])
def test_gpu_matches_cpu_laspack(libs, it, pc, sym):
    gpu, cpu = libs
    A = fv_like(8, not sym, seed=5)
    b = np.random.default_rng(6).standard_normal(len(A))
    eps, omega = 1e-10, 1.2
    xg, ig, ag = _solve(gpu, it, pc, A, b, sym, eps, omega)
    xc, ic, ac = _solve(cpu, it, pc, A, b, sym, eps, omega)
    assert ag < eps and ac < eps
    assert abs(ig - ic) <= 1, (it, pc, ig, ic)
    assert np.linalg.norm(xg - xc) <= 1e-8 * np.linalg.norm(xc)
    r = b - A @ xg
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2 * eps


@pytest.mark.parametrize("pc", ["JacobiPrecond", "SSORPrecond", "ILUPrecond"])
def test_preconditioner_entry_points(libs, pc):
    """y = M^-1 c applied once, GPU against the CPU restatement."""
    gpu, cpu = libs
    A = fv_like(6, True, seed=9)
    c = np.random.default_rng(10).standard_normal(len(A))
    ys = []
    for L in (gpu, cpu):
        q = _load(L, A, False)
        y, cc = _vec(L, np.zeros(len(c))), _vec(L, c)
        getattr(L, pc)(C.byref(q), C.byref(y), C.byref(cc), 1.3)
        ys.append(np.array([y.Cmp[i + 1] for i in range(len(c))]))
        L.Q_Destr(C.byref(q))
    assert np.linalg.norm(ys[0] - ys[1]) <= 1e-12 * np.linalg.norm(ys[1])


def _csr(A):
    rp, cl, vl = [0], [], []
    for i in range(len(A)):
        js = np.nonzero(A[i])[0]
        cl += list(js)
        vl += list(A[i, js])
        rp.append(len(cl))
    return np.array(rp, np.int32), np.array(cl, np.int32), np.array(vl)


@pytest.mark.parametrize("method,precond", [("GMRES", "SSOR"), ("GMRES", "ILU"), ("GMRES", "none"),
                                            ("CG", "SSOR"), ("CG", "ILU")])
def test_csr_abi_general_solvers(method, precond):
    sym = method == "CG"
    A = fv_like(10, not sym, seed=3)
    rp, cl, vl = _csr(A)
    b = np.random.default_rng(4).standard_normal(len(A))
    x, it, res, st = csr_solve(rp, cl, vl, b, None, method=method, precond=precond, maxit=3000, eps=1e-10,
                               omega=1.3)
    assert st == 0 and res < 1e-10 and it > 0
    xs = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xs) <= 1e-7 * np.linalg.norm(xs)


@pytest.mark.parametrize("name", ["cavity_hex6_tight", "cavity_tet_tight", "cht_ke_tight"])
def test_reference_solver_mode_fields(name):
    """GMRES + SSOR / CG + SSOR as the reference calls them, tight tolerance: the
    reference's fields within relative L2 1e-10 (the fixtures' Krylov method does
    not matter at this tolerance)."""
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    mesh, rows, iters, env = make_golden.cases()[name]
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mesh, rows)
        with NavierStokesSolver(p, {"rtc": float(env["SYSU_ORACLE_RTC"]), "reference_solvers": 1}) as s:
            assert s.get_option("mom.kind") == 2 and s.get_option("p.precond") == 2
            s.iterate(iters)
            for f in ("U", "V", "W", "P", "T", "TE", "ED"):
                if "fields_" + f not in gold.files:
                    continue
                r = gold["fields_" + f]
                a = s.get(f)
                e = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-300)
                assert e < 1e-10, (name, f, e)

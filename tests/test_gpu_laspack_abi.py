"""GPU tests of the LASPack-compatible C ABI (include/laspack/laspack.h).

1. Direct calls through ctypes: Q_Constr/Q_SetLen/Q_SetEntry with upper-triangle
   storage for a symmetric matrix, CGIter / BiCGSTABIter / GMRESIter, RTC queries.
2. The reference's own, unmodified sources linked against libsysucfd.so
   (oracle/_ref/cycas_ref_gpulaspack) against the same sources linked against the
   CPU LASPack restatement (oracle/_ref/cycas_ref): same fields after N iterations.
"""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

import make_golden
from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300._lib import LIB_PATH

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class Vec(C.Structure):
    _fields_ = [("Name", C.c_char_p), ("Dim", C.c_size_t), ("Instance", C.c_int), ("OwnData", C.c_int),
                ("Cmp", C.POINTER(C.c_double))]


class QMat(C.Structure):
    _fields_ = [("Name", C.c_char_p), ("Dim", C.c_size_t), ("Symmetry", C.c_int), ("ElOrder", C.c_int),
                ("Instance", C.c_int), ("OwnData", C.c_int), ("Len", C.c_void_p), ("El", C.c_void_p),
                ("Priv", C.c_void_p)]


@pytest.fixture(scope="module")
def las():
    L = C.CDLL(LIB_PATH)
    L.Q_Constr.argtypes = [C.POINTER(QMat), C.c_char_p, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int]
    L.Q_SetLen.argtypes = [C.POINTER(QMat), C.c_size_t, C.c_size_t]
    L.Q_SetEntry.argtypes = [C.POINTER(QMat), C.c_size_t, C.c_size_t, C.c_size_t, C.c_double]
    L.Q_Destr.argtypes = [C.POINTER(QMat)]
    L.V_Constr.argtypes = [C.POINTER(Vec), C.c_char_p, C.c_size_t, C.c_int, C.c_int]
    L.SetRTCAccuracy.argtypes = [C.c_double]
    L.GetLastAccuracy.restype = C.c_double
    for it in ("CGIter", "BiCGSTABIter", "GMRESIter"):
        getattr(L, it).argtypes = [C.POINTER(QMat), C.POINTER(Vec), C.POINTER(Vec), C.c_int, C.c_void_p, C.c_double]
        getattr(L, it).restype = C.POINTER(Vec)
    return L


def laplacian3d(m, shift=0.0):
    n = m ** 3
    A = np.zeros((n, n))
    for i in range(m):
        for j in range(m):
            for k in range(m):
                r = (i * m + j) * m + k
                A[r, r] = 6.0 + shift
                for d in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
                    a, b, c = i + d[0], j + d[1], k + d[2]
                    if 0 <= a < m and 0 <= b < m and 0 <= c < m:
                        A[r, (a * m + b) * m + c] = -1.0
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


@pytest.mark.parametrize("it,sym", [("CGIter", True), ("BiCGSTABIter", False), ("GMRESIter", False)])
def test_laspack_abi_solves_on_gpu(las, it, sym):
    A = laplacian3d(7, 0.05)
    n = len(A)
    if not sym:
        for k in range(n - 1):
            A[k + 1, k] -= 0.5
            A[k + 1, k + 1] += 0.5
    rng = np.random.default_rng(3)
    b = rng.standard_normal(n)
    q = _load(las, A, sym)
    x, bb = _vec(las, np.zeros(n)), _vec(las, b)
    las.SetRTCAccuracy(1e-12)
    getattr(las, it)(C.byref(q), C.byref(x), C.byref(bb), 1000, C.cast(las.SSORPrecond, C.c_void_p), 1.3)
    xs = np.linalg.solve(A, b)
    xg = np.array([x.Cmp[i + 1] for i in range(n)])
    assert np.linalg.norm(xg - xs) / np.linalg.norm(xs) < 1e-9
    assert las.GetLastAccuracy() < 1e-12
    assert 0 < las.GetLastNoIter() < 1000
    las.Q_Destr(C.byref(q))


def _run(exe, d, env):
    os.makedirs(os.path.join(d, "out"), exist_ok=True)
    subprocess.run([exe, "-paramfile", "param.in", "-iters", "10", "-dump", "out", "-quiet"], cwd=d, env=env,
                   check=True, capture_output=True, timeout=600)
    return {f: np.fromfile(os.path.join(d, "out", f + ".f64")) for f in ("U", "V", "W", "P", "RUFace", "T")}


@pytest.mark.parametrize("name", ["cavity_tet_tight", "cht_ke_tight"])
def test_reference_sources_on_gpu_laspack(name):
    cpu = os.path.join(ROOT, "oracle", "_ref", "cycas_ref")
    gpu = os.path.join(ROOT, "oracle", "_ref", "cycas_ref_gpulaspack")
    if not (os.path.exists(cpu) and os.path.exists(gpu)):
        pytest.skip("reference binaries not built (no reference sources installed)")
    mesh, rows, _, _ = make_golden.cases()[name]
    with tempfile.TemporaryDirectory() as a, tempfile.TemporaryDirectory() as b:
        mg.write_case(a, mesh, rows)
        mg.write_case(b, mesh, rows)
        ra = _run(cpu, a, dict(os.environ, SYSU_ORACLE_GMRES_AS="BiCGSTAB", SYSU_ORACLE_SSOR_AS="Jacobi",
                               SYSU_ORACLE_RTC="1e-13"))
        rb = _run(gpu, b, dict(os.environ, SYSU_LASPACK_RTC="1e-13"))
        for f in ra:
            nr = np.linalg.norm(ra[f]) or 1.0
            assert np.linalg.norm(ra[f] - rb[f]) / nr < 1e-10, f

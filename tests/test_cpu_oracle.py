"""CPU tests of the oracle itself (no GPU).

* the numpy restatement (oracle/simple_np.py) against the golden fixtures that the
  compiled reference produced (pinning the restatement to the reference);
* the C restatement of the LASPack API (oracle/laspack_cpu.c) against dense numpy
  solves, its row/entry semantics and its run-time-control (RTC) behaviour.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np
import pytest

import make_golden
from sysu_cfd_heat_gb300 import meshgen as mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import simple_np  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden")
CASES = make_golden.cases()


def rel(a, r):
    nr = np.linalg.norm(r)
    return np.linalg.norm(a - r) / (nr if nr > 0 else 1.0)


@pytest.mark.parametrize("name", [n for n in CASES if not n.startswith("c1_")])
def test_numpy_oracle_matches_reference(name):
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    mesh, rows, iters, env = CASES[name]
    with tempfile.TemporaryDirectory() as tmp:
        s = simple_np.SimpleNP(mg.write_case(tmp, mesh, rows), rtc=float(env["SYSU_ORACLE_RTC"]))
        assert s.iterate(iters) == len(gold["res"])
        np.testing.assert_allclose(s.Residual[:4], gold["res"][-1, 1:5], rtol=1e-9, atol=1e-15)
        fields = [("U", s.U), ("V", s.V), ("W", s.W), ("P", s.P), ("RUFace", s.RUFace), ("TE", s.TE),
                  ("ED", s.ED), ("VisTur", s.VisTur), ("T", s.T)]
        if s.solid is not None:
            fields.append(("solid_T", s.sT))
        for f, a in fields:
            assert rel(a, gold["fields_" + f]) < 1e-11, (name, f, rel(a, gold["fields_" + f]))


@pytest.mark.parametrize("name", ["cavity_hex6_tight", "cavity_tet_tight"])
def test_numpy_oracle_iteration1_systems(name):
    """The restated momentum and p' systems equal the ones the reference handed to LASPack."""
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    mesh, rows, iters, env = CASES[name]
    with tempfile.TemporaryDirectory() as tmp:
        s = simple_np.SimpleNP(mg.write_case(tmp, mesh, rows), rtc=float(env["SYSU_ORACLE_RTC"]))
        s.calculate_velocity()
        n = s.d.nc
        for c in range(3):
            k = f"solve{c}_"
            A = dense(*s.mom_A[:3], n)
            Ar = dense(gold[k + "rowptr"], gold[k + "col"], gold[k + "val"], n)
            assert np.max(np.abs(A - Ar)) <= 1e-13 * np.max(np.abs(Ar))
            assert rel(s.mom_b[c], gold[k + "b"]) < 1e-13
        s.calculate_pressure()
        Ar = dense(gold["solve3_rowptr"], gold["solve3_col"], gold["solve3_val"], n)
        assert np.max(np.abs(dense(*s.p_A[:3], n) - Ar)) <= 1e-13 * np.max(np.abs(Ar))
        assert rel(s.p_b, gold["solve3_b"]) < 1e-12
        assert abs(s.p_iters - int(gold["solve3_iters"])) <= 1


def dense(rp, cl, vl, n):
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            A[i, cl[k]] += vl[k]
    return A


def test_numpy_krylov_on_reference_systems():
    """Restated CG / BiCGSTAB reproduce the reference's solutions of its own systems."""
    gold = np.load(os.path.join(GOLD, "cavity_tet_tight.npz"))
    for k in range(4):
        pre = f"solve{k}_"
        rp, cl, vl = gold[pre + "rowptr"], gold[pre + "col"], gold[pre + "val"]
        n = len(rp) - 1
        diag = np.array([vl[rp[i]:rp[i + 1]][cl[rp[i]:rp[i + 1]] == i].sum() for i in range(n)])
        fn = simple_np.cg if str(gold[pre + "method"]) == "CG" else simple_np.bicgstab
        x, it, res = fn((rp, cl, vl, diag), gold[pre + "b"], gold[pre + "x0"].copy(), int(gold[pre + "maxit"]),
                        float(gold[pre + "eps"]), float(gold[pre + "omega"]))
        assert abs(it - int(gold[pre + "iters"])) <= 1
        assert rel(x, gold[pre + "x"]) < 1e-10


# ---- the C LASPack restatement ------------------------------------------------------
LAS = os.path.join(ROOT, "oracle", "_ref", "liblaspack_cpu.so")


class Vec(C.Structure):
    _fields_ = [("Name", C.c_char_p), ("Dim", C.c_size_t), ("Instance", C.c_int), ("OwnData", C.c_int),
                ("Cmp", C.POINTER(C.c_double))]


class QMat(C.Structure):
    _fields_ = [("Name", C.c_char_p), ("Dim", C.c_size_t), ("Symmetry", C.c_int), ("ElOrder", C.c_int),
                ("Instance", C.c_int), ("OwnData", C.c_int), ("Len", C.c_void_p), ("El", C.c_void_p),
                ("Priv", C.c_void_p)]


@pytest.fixture(scope="module")
def las():
    if not os.path.exists(LAS):
        pytest.skip("oracle/_ref/liblaspack_cpu.so not built (make -C oracle)")
    L = C.CDLL(LAS)
    L.Q_Constr.argtypes = [C.POINTER(QMat), C.c_char_p, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int]
    L.Q_SetLen.argtypes = [C.POINTER(QMat), C.c_size_t, C.c_size_t]
    L.Q_SetEntry.argtypes = [C.POINTER(QMat), C.c_size_t, C.c_size_t, C.c_size_t, C.c_double]
    L.Q_Destr.argtypes = [C.POINTER(QMat)]
    L.V_Constr.argtypes = [C.POINTER(Vec), C.c_char_p, C.c_size_t, C.c_int, C.c_int]
    L.V_Destr.argtypes = [C.POINTER(Vec)]
    L.SetRTCAccuracy.argtypes = [C.c_double]
    L.GetLastAccuracy.restype = C.c_double
    for it in ("CGIter", "BiCGSTABIter", "GMRESIter"):
        getattr(L, it).argtypes = [C.POINTER(QMat), C.POINTER(Vec), C.POINTER(Vec), C.c_int, C.c_void_p, C.c_double]
        getattr(L, it).restype = C.POINTER(Vec)
    return L


def _load(L, A, symmetric=False):
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


def _get(x, n):
    return np.array([x.Cmp[i + 1] for i in range(n)])


def laplacian2d(m, shift=0.0):
    n = m * m
    A = np.zeros((n, n))
    for i in range(m):
        for j in range(m):
            k = i * m + j
            A[k, k] = 4.0 + shift
            for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                if 0 <= i + di < m and 0 <= j + dj < m:
                    A[k, (i + di) * m + j + dj] = -1.0
    return A


@pytest.mark.parametrize("pc", ["JacobiPrecond", "SSORPrecond", "ILUPrecond", None])
def test_laspack_cg_symmetric_upper_storage(las, pc):
    A = laplacian2d(8, 0.1)
    n = len(A)
    rng = np.random.default_rng(1)
    b = rng.standard_normal(n)
    q = _load(las, A, symmetric=True)
    x, bb = _vec(las, np.zeros(n)), _vec(las, b)
    las.SetRTCAccuracy(1e-12)
    pcf = C.cast(getattr(las, pc), C.c_void_p) if pc else None
    las.CGIter(C.byref(q), C.byref(x), C.byref(bb), 500, pcf, 1.2)
    xs = np.linalg.solve(A, b)
    assert np.linalg.norm(_get(x, n) - xs) / np.linalg.norm(xs) < 1e-10
    assert las.GetLastAccuracy() < 1e-12
    assert 0 < las.GetLastNoIter() < 500
    las.Q_Destr(C.byref(q))


@pytest.mark.parametrize("it", ["BiCGSTABIter", "GMRESIter"])
@pytest.mark.parametrize("pc", ["JacobiPrecond", "SSORPrecond", "ILUPrecond"])
def test_laspack_nonsymmetric(las, it, pc):
    A = laplacian2d(7, 0.5)
    n = len(A)
    for k in range(n - 1):  # upwind convection makes it non-symmetric
        A[k + 1, k] -= 0.8
        A[k + 1, k + 1] += 0.8
    rng = np.random.default_rng(2)
    b = rng.standard_normal(n)
    q = _load(las, A)
    x, bb = _vec(las, rng.standard_normal(n)), _vec(las, b)
    las.SetRTCAccuracy(1e-11)
    getattr(las, it)(C.byref(q), C.byref(x), C.byref(bb), 500, C.cast(getattr(las, pc), C.c_void_p), 1.0)
    xs = np.linalg.solve(A, b)
    assert np.linalg.norm(_get(x, n) - xs) / np.linalg.norm(xs) < 1e-8
    r = b - A @ _get(x, n)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-10
    las.Q_Destr(C.byref(q))


def test_laspack_row_reset_and_maxiter(las):
    """Q_SetLen on an assembled row replaces it (navier_scalar.cpp:135-136), and an
    unreachable tolerance stops at MaxIter with the reached accuracy reported."""
    A = laplacian2d(6)
    n = len(A)
    q = _load(las, A)
    las.Q_SetLen(C.byref(q), 3, 1)
    las.Q_SetEntry(C.byref(q), 3, 0, 3, 1.0)
    A2 = A.copy()
    A2[2, :] = 0.0
    A2[2, 2] = 1.0
    b = np.ones(n)
    x, bb = _vec(las, np.zeros(n)), _vec(las, b)
    las.SetRTCAccuracy(1e-30)
    las.BiCGSTABIter(C.byref(q), C.byref(x), C.byref(bb), 7, C.cast(las.JacobiPrecond, C.c_void_p), 1.0)
    assert las.GetLastNoIter() == 7
    acc = las.GetLastAccuracy()
    r = np.linalg.norm(b - A2 @ _get(x, n)) / np.linalg.norm(b)
    assert abs(acc - r) < 1e-12 + 1e-6 * r
    las.Q_Destr(C.byref(q))


def test_laspack_zero_rhs_converges_immediately(las):
    A = laplacian2d(4)
    n = len(A)
    q = _load(las, A)
    x, bb = _vec(las, np.zeros(n)), _vec(las, np.zeros(n))
    las.SetRTCAccuracy(1e-8)
    las.GMRESIter(C.byref(q), C.byref(x), C.byref(bb), 500, C.cast(las.SSORPrecond, C.c_void_p), 1.2)
    assert las.GetLastNoIter() == 0
    assert np.all(_get(x, n) == 0.0)
    las.Q_Destr(C.byref(q))


@pytest.mark.parametrize("mesh", ["tet", "hex"])
def test_lsq_gradient_restatement_exact_for_linear_fields(mesh):
    """The least-squares gradient (an option of this implementation; the reference
    has Green-Gauss only) is exact for a linear field with consistent boundary
    values on any mesh: pins the restatement the GPU kernel is checked against."""
    m = mg.lid_cavity_tet(5, 5, 4, jitter=0.2, seed=3) if mesh == "tet" else mg.lid_cavity_hex(6)
    with tempfile.TemporaryDirectory() as tmp:
        s = simple_np.SimpleNP(mg.write_case(tmp, m, mg.cavity_param("x", 2, mu=0.01)))
        d = s.d
        a = np.array([1.5, -2.0, 0.75])
        phi = 3.0 + d.g.cx @ a
        bphi = 3.0 + d.g.fx[d.m.bface] @ a
        gr = d.gradient_lsq(phi, bphi)
        np.testing.assert_allclose(gr, np.broadcast_to(a, gr.shape), rtol=0, atol=1e-10)

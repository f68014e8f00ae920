"""GPU parity of the SIMPLE hot path against the reference (through the C ABI).

The fixtures in tests/golden were produced by the reference's own C++ (oracle/_ref,
see make_golden.py) on the same seeded meshes; the GPU path runs the same solver
choices (BiCGSTAB + Jacobi at the GMRES call sites, CG + Jacobi for p') and tolerances.

Tolerances (relative L2):
* 1e-10 for the plain FP64 path with inner tolerance 1e-13 (``*_tight`` cases);
* 1e-6 for configuration 1 (24^3 cavity, 300 iterations, inner tolerance 1e-8), where
  the two codes stop their Krylov solves at different 1e-8-level iterates.
"""
import os
import tempfile

import numpy as np
import pytest

import make_golden
from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.solver import NavierStokesSolver, csr_solve, csr_spmv

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = make_golden.cases()


def rel(a, r):
    nr = np.linalg.norm(r)
    return np.linalg.norm(a - r) / (nr if nr > 0 else 1.0)


def make_solver(name, tmp):
    mesh, rows, iters, env = CASES[name]
    p = mg.write_case(tmp, mesh, rows)
    s = NavierStokesSolver(p, {"rtc": float(env["SYSU_ORACLE_RTC"])})
    return s, iters


CELL_FIELDS = ["U", "V", "W", "P", "Apr", "TE", "ED", "VisTur", "T"]
FACE_FIELDS = ["RUFace", "BU", "BV", "BW", "BRo", "BTE", "BED", "BTem", "Bq"]


@pytest.mark.parametrize("name", [n for n in CASES if n.endswith("_tight") or n.endswith("_weno")
                                  or n.endswith("_barth") or n.endswith("_mlp")])
def test_fields_match_reference(name):
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    with tempfile.TemporaryDirectory() as tmp:
        s, iters = make_solver(name, tmp)
        with s:
            done = s.iterate(iters)
            assert done == len(gold["res"])
            res = s.Residual
            np.testing.assert_allclose(res[:4], gold["res"][-1, 1:5], rtol=1e-7, atol=1e-14)
            names = CELL_FIELDS + FACE_FIELDS
            if "solid_T" in gold.files:
                names += ["solid_T", "solid_Bq", "solid_BTem"]
            for f in names:
                if "fields_" + f not in gold.files:
                    continue
                r = gold["fields_" + f]
                a = s.get(f)
                assert rel(a, r) < 1e-10, (name, f, rel(a, r))


def test_config1_cavity24():
    gold = np.load(os.path.join(GOLD, "c1_cavity24.npz"))
    with tempfile.TemporaryDirectory() as tmp:
        s, iters = make_solver("c1_cavity24", tmp)
        with s:
            assert s.iterate(iters) == 300
            for f in ("U", "V", "W", "P", "RUFace"):
                e = rel(s.get(f), gold["fields_" + f])
                assert e < 1e-6, (f, e)


@pytest.mark.parametrize("name", ["cavity_hex6_tight", "cavity_tet_tight"])
def test_iteration1_intermediates(name):
    """Gradients, Apr, momentum and p' systems and corrections of iteration 1."""
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    with tempfile.TemporaryDirectory() as tmp:
        s, _ = make_solver(name, tmp)
        with s:
            s.CalculateVelocity()
            s.check()
            for f, g in (("dUdX", "dUdX"), ("dVdX", "dVdX"), ("dWdX", "dWdX"), ("dPdX", "dPdX"), ("Apr", "Apr"),
                         ("U", "Ustar"), ("V", "Vstar"), ("W", "Wstar")):
                assert rel(s.get(f), gold["stage1_" + g]) < 1e-10, (f, rel(s.get(f), gold["stage1_" + g]))
            # momentum matrix and right-hand sides vs the reference's first three solves
            rp, cl, vl = s.matrix("mom")
            b3 = s.get("b3")
            n = len(rp) - 1
            for c in range(3):
                k = f"solve{c}_"
                assert str(gold[k + "method"]) == "BiCGSTAB"
                A_ref = dense(gold[k + "rowptr"], gold[k + "col"], gold[k + "val"], n)
                A_gpu = dense(rp, cl, vl, n)
                assert np.max(np.abs(A_gpu - A_ref)) <= 1e-12 * np.max(np.abs(A_ref))
                assert rel(b3[c * n:(c + 1) * n], gold[k + "b"]) < 1e-12
            s.CalculatePressure()
            s.check()
            k = "solve3_"
            assert str(gold[k + "method"]) == "CG"
            rp, cl, vl = s.matrix("p")
            A_ref = dense(gold[k + "rowptr"], gold[k + "col"], gold[k + "val"], n)
            assert np.max(np.abs(dense(rp, cl, vl, n) - A_ref)) <= 1e-11 * np.max(np.abs(A_ref))
            assert rel(s.get("bp"), gold[k + "b"]) < 1e-10
            for f, g in (("dp", "dp"), ("dPdX", "dPdX_dp"), ("P", "P1"), ("U", "U1"), ("V", "V1"), ("W", "W1"),
                         ("RUFace", "RUFace1")):
                assert rel(s.get(f), gold["stage1_" + g]) < 1e-9, (f, rel(s.get(f), gold["stage1_" + g]))


def dense(rp, cl, vl, n):
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            A[i, cl[k]] += vl[k]
    return A


@pytest.mark.parametrize("name,k", [("cavity_hex6_tight", 0), ("cavity_hex6_tight", 3), ("cavity_tet_tight", 3),
                                    ("cht_ke_tight", 0)])
def test_krylov_on_reference_systems(name, k):
    """The GPU Krylov kernels on the linear systems the reference solved."""
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    pre = f"solve{k}_"
    rp, cl, vl = gold[pre + "rowptr"], gold[pre + "col"], gold[pre + "val"]
    b, x0, xr = gold[pre + "b"], gold[pre + "x0"], gold[pre + "x"]
    method = str(gold[pre + "method"])
    x, it, res, st = csr_solve(rp, cl, vl, b, x0, method=method, precond="Jacobi", maxit=int(gold[pre + "maxit"]),
                               eps=float(gold[pre + "eps"]), omega=float(gold[pre + "omega"]))
    assert st == 0, (st, it, res)
    assert res < float(gold[pre + "eps"])
    assert abs(it - int(gold[pre + "iters"])) <= 2, (it, int(gold[pre + "iters"]))
    # same algorithm, same tolerance: the solutions agree to the tolerance
    assert rel(x, xr) < 1e-9
    y = csr_spmv(rp, cl, vl, x)
    assert np.linalg.norm(b - y) / np.linalg.norm(b) < 10 * float(gold[pre + "eps"])


def test_batched_momentum_equals_separate_solves():
    """u, v, w as one 3-RHS BiCGSTAB launch give the same iterates as three solves."""
    outs = []
    for batched in (1, 0):
        with tempfile.TemporaryDirectory() as tmp:
            s, _ = make_solver("cavity_tet_tight", tmp)
            with s:
                s.set_option("mom_batched", batched)
                s.iterate(3)
                outs.append([s.get(f) for f in ("U", "V", "W", "P")] + [s.solve_stats()["mom"]["iters"]])
    for a, b in zip(outs[0][:4], outs[1][:4]):
        np.testing.assert_array_equal(a, b)
    assert outs[0][4] == outs[1][4]


def test_deterministic():
    """Two runs are bit-identical (fixed-order reductions, no float atomics)."""
    outs = []
    for _ in range(2):
        with tempfile.TemporaryDirectory() as tmp:
            s, _ = make_solver("cht_ke_tight", tmp)
            with s:
                s.iterate(4)
                outs.append([s.get(f) for f in ("U", "P", "TE", "ED", "T", "solid_T")])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)

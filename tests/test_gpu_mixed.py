"""GPU tests of the mixed-precision form: FP32 inner Jacobi-CG in FP64 defect correction.

The form stops on the FP64 residual ||b - A x|| / ||b|| < eps, the same test as the FP64
CG, so on one linear system the two agree to the tolerance; over a SIMPLE run the fields
agree at convergence within 1e-6 relative L2 (the bar for the mixed form).
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


def rel(a, r):
    return np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-300)


@pytest.mark.parametrize("name", ["cavity_hex6_tight", "cavity_tet_tight"])
@pytest.mark.parametrize("eps", [1e-8, 1e-12])
def test_mixed_cg_on_reference_p_system(name, eps):
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    pre = "solve3_"
    rp, cl, vl, b = gold[pre + "rowptr"], gold[pre + "col"], gold[pre + "val"], gold[pre + "b"]
    x64, it64, res64, st64 = csr_solve(rp, cl, vl, b, None, method="CG", maxit=5000, eps=eps, omega=1.3)
    xm, itm, resm, stm = csr_solve(rp, cl, vl, b, None, method="CG-mixed", maxit=5000, eps=eps, omega=1.3)
    assert st64 == 0 and stm == 0
    assert resm < eps
    # the reported residual is the true FP64 residual
    r = b - csr_spmv(rp, cl, vl, xm)
    assert abs(np.linalg.norm(r) / np.linalg.norm(b) - resm) <= 1e-3 * resm + 1e-16
    # p' is defined up to a constant on a closed cavity: compare against the reference cell
    d64 = x64 - x64[0]
    dm = xm - xm[0]
    assert rel(dm, d64) < 50 * eps / 1e-8 * 1e-6 + 1e-9


def test_mixed_c1_fields_at_convergence():
    """Configuration 1 (24^3 cavity, 300 iterations) with the mixed p' solve."""
    gold = np.load(os.path.join(GOLD, "c1_cavity24.npz"))
    mesh, rows, iters, env = make_golden.cases()["c1_cavity24"]
    with tempfile.TemporaryDirectory() as tmp:
        with NavierStokesSolver(mg.write_case(tmp, mesh, rows), {"rtc": 1e-8, "p.mixed": 1}) as s:
            assert s.iterate(iters) == iters
            for f in ("U", "V", "W", "P"):
                e = rel(s.get(f), gold["fields_" + f])
                assert e < 1e-6, (f, e)

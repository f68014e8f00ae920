"""Mixed-precision BiCGSTAB: FP32 inner iterations in FP64 defect correction.

On one linear system it stops on the same FP64 residual test as the FP64
BiCGSTAB (||b - A x|| / ||b|| < eps, the reported residual is the true one), so
the two solutions agree to the conditioning times eps.  In the SIMPLE loop the
k, eps, T (and p', solid T) solves of the CHT k-eps channel in the mixed form
reach the FP64 form's steady fields within 1e-6 relative L2, the bar the mixed
form is held to.
"""
import os
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.solver import NavierStokesSolver, SysuError, csr_solve, csr_spmv

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _convection_diffusion(nx, ny, nz, peclet, seed):
    """Upwind convection-diffusion on a box grid: non-symmetric, an M-matrix."""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    idx = np.arange(n).reshape(nz, ny, nx)
    rows, cols, vals = [], [], []
    for d, (axis, vel) in enumerate(((2, 1.0), (1, 0.5), (0, -0.3))):
        lo = np.take(idx, range(0, idx.shape[axis] - 1), axis=axis).ravel()
        hi = np.take(idx, range(1, idx.shape[axis]), axis=axis).ravel()
        w = 1.0 + 0.2 * rng.random(lo.size)
        c = peclet * vel
        # flux lo -> hi (upwind): the upstream cell feeds the downstream one
        a_lohi = -(w + max(-c, 0.0))
        a_hilo = -(w + max(c, 0.0))
        rows += [lo, hi]
        cols += [hi, lo]
        vals += [a_lohi, a_hilo]
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
    return np.cumsum(rp).astype(np.int32), cols.astype(np.int32), vals, rng.standard_normal(n)


@pytest.mark.parametrize("peclet", [0.5, 4.0])
@pytest.mark.parametrize("eps", [1e-8, 1e-12])
def test_mixed_bicgstab_matches_fp64(peclet, eps):
    rp, cl, vl, b = _convection_diffusion(24, 20, 16, peclet, seed=3)
    x64, it64, res64, st64 = csr_solve(rp, cl, vl, b, method="BiCGSTAB", precond="Jacobi", maxit=5000, eps=eps)
    xm, itm, resm, stm = csr_solve(rp, cl, vl, b, method="BiCGSTAB-mixed", precond="Jacobi", maxit=5000, eps=eps)
    assert st64 == 0 and stm == 0, (st64, stm)
    assert resm < eps
    r = b - csr_spmv(rp, cl, vl, xm)
    true = np.linalg.norm(r) / np.linalg.norm(b)
    assert true < eps and abs(true - resm) <= 1e-3 * resm + 1e-18
    assert _rel(xm, x64) < 1e3 * eps


def test_mixed_bicgstab_on_reference_momentum_system():
    gold = np.load(os.path.join(GOLD, "cavity_hex6_tight.npz"))
    pre = "solve0_"  # the u-momentum system of outer iteration 1, as the reference assembled it
    rp, cl, vl, b = gold[pre + "rowptr"], gold[pre + "col"], gold[pre + "val"], gold[pre + "b"]
    x64, _, _, st64 = csr_solve(rp, cl, vl, b, method="BiCGSTAB", precond="Jacobi", maxit=2000, eps=1e-12)
    xm, _, resm, stm = csr_solve(rp, cl, vl, b, method="BiCGSTAB-mixed", precond="Jacobi", maxit=2000, eps=1e-12)
    assert st64 == 0 and stm == 0 and resm < 1e-12
    assert _rel(xm, x64) < 1e-9


def test_mixed_bicgstab_no_preconditioner_and_zero_rhs():
    rp, cl, vl, b = _convection_diffusion(10, 8, 6, 1.0, seed=5)
    xm, _, resm, stm = csr_solve(rp, cl, vl, b, method="BiCGSTAB-mixed", precond="none", maxit=3000, eps=1e-10)
    assert stm == 0 and resm < 1e-10
    x0, it0, res0, st0 = csr_solve(rp, cl, vl, np.zeros_like(b), method="BiCGSTAB-mixed", precond="Jacobi")
    assert st0 == 0 and it0 == 0 and not x0.any()


def test_simple_scalars_mixed_reach_fp64_steady_state():
    """Each form runs until its outer residuals are below 1e-11, as NSSolve stops
    on its convergence criterion.  (Further on, at the round-off floor, the p'
    right-hand side of this closed-pressure channel is round-off noise: zero in
    the FP64 run, an inconsistent right-hand side of the singular p' system in
    the mixed run, which no CG solves -- runs stop before that.)"""
    iters = 200
    with tempfile.TemporaryDirectory() as d:
        p = mg.write_case(d, mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", iters + 1, turb=True))
        out = {}
        forms = (("fp64", {}), ("mixed", {"p.mixed": 1, "ke.mixed": 1, "t.mixed": 1, "ts.mixed": 1}))
        for name, opts in forms:
            o = {"rtc": 1e-12}
            o.update(opts)
            with NavierStokesSolver(p, o) as s:
                done = 0
                while done < iters and (done == 0 or not max(s.Residual) < 1e-11):
                    s.iterate(5)
                    done += 5
                assert max(s.Residual) < 1e-11, (name, done, s.Residual)
                if name == "mixed":
                    st = s.solve_stats()
                    assert st["k"]["status"][0] == 0 and st["T"]["status"][0] == 0, st
                out[name] = {f: s.get(f) for f in ("U", "V", "W", "P", "T", "TE", "ED", "VisTur", "solid_T")}
        for f, ref in out["fp64"].items():
            e = _rel(out["mixed"][f], ref)
            assert e < 1e-6, (f, e)


def test_mixed_option_rules():
    with tempfile.TemporaryDirectory() as d:
        p = mg.write_case(d, mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", 2, turb=True))
        with NavierStokesSolver(p, {}) as s:
            s.set_option("mom.mixed", 1)  # BiCGSTAB momentum: allowed
            s.set_option("mom.mixed", 0)
            s.set_option("mom.kind", 2)   # GMRES has no mixed form
            with pytest.raises(SysuError):
                s.set_option("mom.mixed", 1)
            s.set_option("mom.kind", 1)
            s.set_option("ke.mixed", 1)
            with pytest.raises(SysuError):
                s.set_option("scalars_batched", 1)
            s.set_option("ke.mixed", 0)
            s.set_option("scalars_batched", 1)
            with pytest.raises(SysuError):
                s.set_option("t.mixed", 1)


@pytest.mark.parametrize("batched", [1, 0])
def test_momentum_mixed_reaches_the_fp64_fields(batched):
    """Option mom.mixed: u, v and w by BiCGSTAB with FP32 recurrences -- together on
    interleaved vectors with FP64 residual replacement (mom_batched 1), or one after
    another with FP32 inner iterations in FP64 defect correction (mom_batched 0);
    solved to a tight tolerance, the SIMPLE fields equal the FP64 form's."""
    import tempfile

    from sysu_cfd_heat_gb300 import meshgen as mg
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_tet(8, 8, 6, jitter=0.2), mg.cavity_param("x", 20, mu=0.0025))
        out = {}
        for name, opts in (("fp64", {}), ("mixed", {"mom.mixed": 1, "p.mixed": 1, "mom_batched": batched})):
            with NavierStokesSolver(p, dict({"rtc": 1e-11}, **opts)) as s:
                assert s.iterate(15) == 15
                st = s.solve_stats()["mom"]
                assert all(v == 0 for v in st["status"]), st
                out[name] = {f: s.get(f) for f in ("U", "V", "W", "P")}
    for f, a in out["mixed"].items():
        r = out["fp64"][f]
        assert np.linalg.norm(a - r) / np.linalg.norm(r) < 1e-8, f

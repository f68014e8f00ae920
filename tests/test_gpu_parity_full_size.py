"""Parity at the benchmark configurations' own sizes, against the reference binary.

The golden fixtures of test_gpu_parity.py hold meshes of at most 13,824 cells, and at
size the GPU kernels run other instantiations (the p' CG switches to wider tiles and
more of them per CTA at 1M rows, the grids of the BiCGSTAB grow with n).  Here the
compiled reference (oracle/_ref/cycas_ref: the reference's src/*.cpp, unmodified, with
the LASPack restatement) and the GPU path run the same two full-size cases:

* configuration 3: the 1,996,800-cell jittered-tet lid cavity (80 x 80 x 52 hexes x 6
  tets, seed 20261203, Re 400) for 2 outer iterations (navier.cpp:33-68);
* configuration 2: the k-epsilon conjugate-heat-transfer channel, 256,000 fluid +
  51,200 solid hexes, for 5 outer iterations (navier_scalar.cpp:14-172,
  HeatConductionSolver.cpp:47-223), without the volumetric solid source, which the
  reference cannot express (the GPU path's option ``solid_source`` stays 0), and from
  a fluid at rest (see below).

Both codes remap the reference's GMRES + SSOR call sites to BiCGSTAB + Jacobi and CG +
SSOR to CG + Jacobi, and solve every system to a relative residual of 1e-13, where
the solutions are unique to ~1e-13 and the fields cannot depend on the Krylov
internals.  Configuration 3 lifts every iteration cap (its p' solve needs ~2,000 CG
iterations to 1e-13; the reference's cap is 1,000), and so does configuration 2.

Configuration 2 starts with the fluid at rest (the inlet still at 1 m/s) instead of
the bench's uniform 1 m/s everywhere.  From the uniform start the first p' right-hand
side is round-off (the flow conserves mass to ~1e-19): no solve reaches 1e-13
relative to it, the pure-Neumann p' matrix is singular only up to rounding, and the
capped CG drifts along its near-null vector by an amount set by where it stops.  The
reference's own residual monitors after 4 iterations move by 10 % between caps of
3,000 and 5,000 iterations there, so no code can match it.  From rest every solve has
a real right-hand side and converges (~800 CG iterations to 1e-13), and the
reference's fields do not depend on the cap at all.

Tolerance: relative L2 1e-10 per field, the same bar as the small golden cases, for
configuration 3.  In configuration 2 the k-epsilon wall functions and the interface
heat flux make the reference's own fields sensitive to its inner tolerance: between
1e-12 and 1e-13 they move by 1e-9 (U) to 1.2e-7 (Apr), measured here by running the
reference at both.  Each field there is held to max(1e-10, a tenth of that spread of
the reference itself); measured on a GB300, the GPU path differs from the reference
by 4e-14 (solid T) to 1.3e-9 (W), 20 to 800 times below the spread.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.solver import NavierStokesSolver

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "cycas_ref")
REMAP = {"SYSU_ORACLE_GMRES_AS": "BiCGSTAB", "SYSU_ORACLE_SSOR_AS": "Jacobi", "SYSU_ORACLE_RTC": "1e-13"}
RTC = 1e-13
TOL = 1e-10


def _start_reference(case, iters, maxit, rtc="1e-13", out="out"):
    os.makedirs(os.path.join(case, out), exist_ok=True)
    env = dict(os.environ, SYSU_ORACLE_MAXIT=str(maxit), **REMAP)
    env["SYSU_ORACLE_RTC"] = rtc
    cmd = [REF_BIN, "-paramfile", "param.in", "-iters", str(iters), "-dump", out, "-quiet"]
    return subprocess.Popen(cmd, cwd=case, env=env, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)


def _finish_reference(p, case, fields, out="out"):
    _, err = p.communicate(timeout=1500)
    assert p.returncode == 0, err.decode()[-2000:]
    res = np.loadtxt(os.path.join(case, out, "iters.txt"), ndmin=2)
    return res, {f: np.fromfile(os.path.join(case, out, f + ".f64")) for f in fields
                 if os.path.exists(os.path.join(case, out, f + ".f64"))}


def _rel(a, r):
    nr = np.linalg.norm(r)
    return float(np.linalg.norm(a - r) / (nr if nr > 0 else 1.0))


def _compare(s, ref, bars=None):
    errs = {}
    for f, r in ref.items():
        a = s.get(f)
        assert a.shape == r.shape, (f, a.shape, r.shape)
        errs[f] = _rel(a, r)
    print("relative L2 vs reference:", errs)
    bad = {f: (e, (bars or {}).get(f, TOL)) for f, e in errs.items() if not e < (bars or {}).get(f, TOL)}
    assert not bad, bad
    return errs


def _gpu(param, iters, maxit):
    s = NavierStokesSolver(param, {"rtc": RTC})
    for eq in ("mom", "p", "ke", "t", "ts"):
        s.set_option(eq + ".maxit", maxit)
    done = s.iterate(iters)
    assert done == iters, done
    return s


def test_config3_two_million_cell_tet_cavity_matches_reference():
    if not os.path.exists(REF_BIN):
        pytest.skip("oracle/_ref/cycas_ref not built (no reference sources installed)")
    fields = ["U", "V", "W", "P", "Apr", "RUFace", "BU", "BV", "BW", "BPre", "dPdX"]
    with tempfile.TemporaryDirectory() as case:
        mesh = mg.lid_cavity_tet(80, 80, 52, jitter=0.2, seed=20261203)
        param = mg.write_case(case, mesh, mg.cavity_param("x", 2, mu=0.0025, urf=(0.7, 0.3, 0.8)))
        del mesh
        p = _start_reference(case, 2, 100000)
        try:
            with _gpu(param, 2, 100000) as s:
                info = s.info()
                assert info["Ncel"] == 1996800
                res_ref, ref = _finish_reference(p, case, fields)
                np.testing.assert_allclose(s.Residual[:4], res_ref[-1, 1:5], rtol=1e-7, atol=1e-14)
                _compare(s, ref)
        finally:
            for q in (p, locals().get("p12")):
                if q is not None and q.poll() is None:
                    q.kill()


def test_config2_cht_channel_matches_reference():
    if not os.path.exists(REF_BIN):
        pytest.skip("oracle/_ref/cycas_ref not built (no reference sources installed)")
    fields = ["U", "V", "W", "P", "T", "TE", "ED", "VisTur", "Apr", "RUFace", "BU", "BV", "BW", "BTem", "Bq",
              "BTE", "BED", "solid_T", "solid_BTem", "solid_Bq"]
    with tempfile.TemporaryDirectory() as case:
        rows = [r[:4] + (0.0,) + r[5:] if (r[0] == "volumn" and r[2] == "fluid") else r
                for r in mg.cht_param("x", 5, nu=1e-5, k_solid=15.0)]
        param = mg.write_case(case, mg.cht_channel(160, 40, 8, 40), rows)
        p = _start_reference(case, 5, 100000)
        p12 = _start_reference(case, 5, 100000, rtc="1e-12", out="out12")
        try:
            with _gpu(param, 5, 100000) as s:
                info = s.info()
                assert info["Ncel"] == 256000 and info["solid_Ncel"] == 51200
                res_ref, ref = _finish_reference(p, case, fields)
                _, ref12 = _finish_reference(p12, case, fields, out="out12")
                spread = {f: _rel(ref12[f], ref[f]) for f in ref}
                print("reference spread 1e-12 vs 1e-13:", spread)
                np.testing.assert_allclose(s.Residual[:4], res_ref[-1, 1:5], rtol=1e-7, atol=1e-14)
                _compare(s, ref, {f: max(TOL, 0.1 * spread[f]) for f in ref})
        finally:
            for q in (p, locals().get("p12")):
                if q is not None and q.poll() is None:
                    q.kill()

"""Transient SIMPLE against the reference's own NSSolve (navier.cpp:20-90).

The reference binary (oracle/_ref/cycas_ref, -nssolve) and the GPU path run the same
transient cases: Euler and the reference's "Dual" scheme (BDF2 coefficients with both
old levels equal to the last step, SaveTransientOldData navier.cpp:212-229), with the
unsteady terms of momentum, k-epsilon (whose eps source the reference recomputes after
the k solve), fluid energy and solid conduction.  Two outer iterations per time step
(MaxOuterStep 3) keep the per-step break rule out of the comparison.  Inner tolerance
1e-12 (1e-11 for the laminar channel): at 1e-13 some solves of the CHT steps sit at the
round-off floor (the reference's own fields move by 1e-6 in p between 1e-13 and 1e-14),
at 1e-12 the reference is stable to 1e-10.  The solid always steps with the Euler term,
as the reference's does (its TimeScheme is the base-class default, navier.h:29).
Bars: velocity components relative to ||U|| (the spanwise and vertical components are
round-off-sized) and T, k, eps, mu_t, solid T within 1e-9; p within 1e-8 of its (small)
norm.
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
ENV = {"SYSU_ORACLE_GMRES_AS": "BiCGSTAB", "SYSU_ORACLE_SSOR_AS": "Jacobi"}


def _transient(rows, dt, total, scheme, inner):
    out = []
    for r in rows:
        if r[0] == "steady":
            out.append(("transient", dt, total, scheme, inner))
        else:
            out.append(r)
    return out


def _cases():
    """name -> (mesh, param rows, inner tolerance)."""
    return {
        "cavity_euler": (mg.lid_cavity_hex(6), _transient(mg.cavity_param("x", 10, mu=0.01), 0.05, 0.2, "Euler", 3),
                         1e-12),
        "cavity_dual": (mg.lid_cavity_hex(6), _transient(mg.cavity_param("x", 10, mu=0.01), 0.05, 0.2, "Dual", 3),
                        1e-12),
        "cht_ke_dual": (mg.cht_channel(8, 4, 2, 3),
                        _transient(mg.cht_param("x", 10, turb=True), 0.01, 0.03, "Dual", 3), 1e-12),
        "cht_ke_euler": (mg.cht_channel(8, 4, 2, 3),
                         _transient(mg.cht_param("x", 10, turb=True), 0.01, 0.03, "Euler", 3), 1e-12),
        # laminar: at 1e-12 the reference's pressure CG stalls above the
        # tolerance and exits (navier_pressure.cpp:30-34), at 1e-13 its p moves by 4e-7
        "cht_lam_euler": (mg.cht_channel(8, 4, 2, 3),
                          _transient(mg.cht_param("x", 10, turb=False), 0.01, 0.03, "Euler", 3), 1e-11),
    }


@pytest.mark.parametrize("name", sorted(_cases()))
def test_transient_matches_reference(name):
    if not os.path.exists(REF_BIN):
        pytest.skip("oracle/_ref/cycas_ref not built (no reference sources installed)")
    mesh, rows, rtc = _cases()[name]
    with tempfile.TemporaryDirectory() as a, tempfile.TemporaryDirectory() as b:
        mg.write_case(a, mesh, rows)
        os.makedirs(os.path.join(a, "out"))
        os.makedirs(os.path.join(a, "tec"))
        subprocess.run([REF_BIN, "-paramfile", "param.in", "-nssolve", "-dump", "out", "-quiet"], cwd=a,
                       env=dict(os.environ, SYSU_ORACLE_RTC=repr(rtc), **ENV), check=True, capture_output=True, timeout=600)
        p = mg.write_case(b, mesh, rows)
        with NavierStokesSolver(p, {"rtc": rtc, "output": 1}) as s:
            done = s.NSSolve()
            assert done > 0
            ref = {f: np.fromfile(os.path.join(a, "out", f + ".f64"))
                   for f in ["U", "V", "W", "P", "T", "TE", "ED", "VisTur"]}
            got = {f: s.get(f) for f in ref}
            unorm = np.linalg.norm(ref["U"])
            errs = {f: np.linalg.norm(got[f] - ref[f]) / unorm for f in ("U", "V", "W")}
            for f in ("P", "T", "TE", "ED", "VisTur"):
                errs[f] = np.linalg.norm(got[f] - ref[f]) / max(np.linalg.norm(ref[f]), 1e-300)
            solid = os.path.join(a, "out", "solid_T.f64")
            if os.path.exists(solid):
                r = np.fromfile(solid)
                errs["solid_T"] = np.linalg.norm(s.get("solid_T") - r) / np.linalg.norm(r)
        # same outer iterations in every time step (tot.dat: time, outIter, averages)
        ta = [l.split()[:2] for l in open(os.path.join(a, "tot.dat")).read().splitlines()[1:]]
        tb = [l.split()[:2] for l in open(os.path.join(b, "tot.dat")).read().splitlines()[1:]]
        assert ta == tb, (ta, tb)
        assert errs["P"] < 1e-8, (name, errs)
        assert max(v for k, v in errs.items() if k != "P") < 1e-9, (name, errs)

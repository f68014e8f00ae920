"""Transient SIMPLE against the reference's own NSSolve (navier.cpp:20-90).

The reference binary (oracle/_ref/cycas_ref, -nssolve) and the GPU path run the same
transient cases: Euler and the reference's "Dual" scheme (BDF2 coefficients with both
old levels equal to the last step, SaveTransientOldData navier.cpp:212-229), with the
unsteady terms of momentum, k-epsilon (whose eps source the reference recomputes after
the k solve), fluid energy and solid conduction.  Two outer iterations per time step
(MaxOuterStep 3) keep the per-step break rule out of the comparison; inner tolerance
1e-13, so the fields after the last step agree within relative L2 1e-10.
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
ENV = {"SYSU_ORACLE_GMRES_AS": "BiCGSTAB", "SYSU_ORACLE_SSOR_AS": "Jacobi", "SYSU_ORACLE_RTC": "1e-13"}


def _transient(rows, dt, total, scheme, inner):
    out = []
    for r in rows:
        if r[0] == "steady":
            out.append(("transient", dt, total, scheme, inner))
        else:
            out.append(r)
    return out


def _cases():
    return {
        "cavity_euler": (mg.lid_cavity_hex(6), _transient(mg.cavity_param("x", 10, mu=0.01), 0.05, 0.2, "Euler", 3)),
        "cavity_dual": (mg.lid_cavity_hex(6), _transient(mg.cavity_param("x", 10, mu=0.01), 0.05, 0.2, "Dual", 3)),
        "cht_ke_dual": (mg.cht_channel(8, 4, 2, 3),
                        _transient(mg.cht_param("x", 10, turb=True), 0.01, 0.03, "Dual", 3)),
        "cht_ke_euler": (mg.cht_channel(8, 4, 2, 3),
                         _transient(mg.cht_param("x", 10, turb=True), 0.01, 0.03, "Euler", 3)),
        "cht_lam_euler": (mg.cht_channel(8, 4, 2, 3),
                          _transient(mg.cht_param("x", 10, turb=False), 0.01, 0.03, "Euler", 3)),
    }


@pytest.mark.parametrize("name", sorted(_cases()))
def test_transient_matches_reference(name):
    if not os.path.exists(REF_BIN):
        pytest.skip("oracle/_ref/cycas_ref not built (no reference sources installed)")
    mesh, rows = _cases()[name]
    with tempfile.TemporaryDirectory() as a, tempfile.TemporaryDirectory() as b:
        mg.write_case(a, mesh, rows)
        os.makedirs(os.path.join(a, "out"))
        os.makedirs(os.path.join(a, "tec"))
        subprocess.run([REF_BIN, "-paramfile", "param.in", "-nssolve", "-dump", "out", "-quiet"], cwd=a,
                       env=dict(os.environ, **ENV), check=True, capture_output=True, timeout=600)
        p = mg.write_case(b, mesh, rows)
        with NavierStokesSolver(p, {"rtc": 1e-13, "output": 1}) as s:
            done = s.NSSolve()
            assert done > 0
            errs = {}
            for f in ["U", "V", "W", "P", "T", "TE", "ED"]:
                ref = np.fromfile(os.path.join(a, "out", f + ".f64"))
                got = s.get(f)
                errs[f] = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
            solid = os.path.join(a, "out", "solid_T.f64")
            if os.path.exists(solid):
                ref = np.fromfile(solid)
                errs["solid_T"] = np.linalg.norm(s.get("solid_T") - ref) / np.linalg.norm(ref)
        # same outer iterations in every time step (tot.dat: time, outIter, averages)
        ta = [l.split()[:2] for l in open(os.path.join(a, "tot.dat")).read().splitlines()[1:]]
        tb = [l.split()[:2] for l in open(os.path.join(b, "tot.dat")).read().splitlines()[1:]]
        assert ta == tb, (ta, tb)
        assert max(errs.values()) < 1e-10, (name, errs)

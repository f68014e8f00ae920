"""Hybrid convection for momentum (option "convection" 1; the reference has only
its upwind scheme with deferred correction): the GPU SIMPLE loop against the
numpy restatement with the same scheme (oracle/simple_np.py, hybrid=True), and a
check that the option changes the solution while option 0 stays the reference's."""
import os
import sys
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.solver import NavierStokesSolver, SysuError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import simple_np  # noqa: E402

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("mesh,mu", [("hex", 0.01), ("tet", 0.002)])
def test_hybrid_matches_oracle(mesh, mu):
    iters = 15
    m = mg.lid_cavity_hex(8) if mesh == "hex" else mg.lid_cavity_tet(5, 5, 4, jitter=0.2, seed=11)
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, m, mg.cavity_param("x", iters + 1, mu=mu))
        ref = simple_np.SimpleNP(p, rtc=1e-12)
        ref.hybrid = True
        assert ref.iterate(iters) == iters
        with NavierStokesSolver(p, {"rtc": 1e-12, "convection": 1}) as s:
            assert s.get_option("convection") == 1
            assert s.iterate(iters) == iters
            for f in ("U", "V", "W"):
                e = _rel(s.get(f), getattr(ref, f))
                assert e < 1e-9, (f, e)
            dp = s.get("P") - s.get("P")[0]
            dr = ref.P - ref.P[0]
            assert _rel(dp, dr) < 1e-8


def test_hybrid_differs_from_default_and_option_checked():
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_hex(8), mg.cavity_param("x", 11, mu=0.002))
        with NavierStokesSolver(p, {"rtc": 1e-10}) as s:
            s.iterate(10)
            u0 = s.get("U")
            s.reset()
            s.set_option("convection", 1)
            s.iterate(10)
            u1 = s.get("U")
            s.reset()
            s.set_option("convection", 0)
            s.iterate(10)
            assert np.array_equal(s.get("U"), u0)
            assert _rel(u1, u0) > 1e-4
            with pytest.raises(SysuError):
                s.set_option("convection", 3)


def test_hybrid_scalars_cht_ke_channel_matches_oracle():
    """k, eps and T convected with the hybrid scheme too (the solid has no convection)."""
    iters = 10
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", iters + 1, turb=True))
        ref = simple_np.SimpleNP(p, rtc=1e-12)
        ref.hybrid = True
        assert ref.iterate(iters) == iters
        with NavierStokesSolver(p, {"rtc": 1e-12, "convection": 1}) as s:
            assert s.iterate(iters) == iters
            pairs = [("U", ref.U), ("V", ref.V), ("W", ref.W), ("TE", ref.TE), ("ED", ref.ED), ("T", ref.T)]
            for f, r in pairs:
                e = _rel(s.get(f), r)
                assert e < 1e-8, (f, e)
            e = _rel(s.get("solid_T"), ref.sT)
            assert e < 1e-8, ("solid_T", e)

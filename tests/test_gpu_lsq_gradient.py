"""Least-squares gradients (option "gradient" 1; the reference has Green-Gauss
only): the GPU gradient of U against the oracle's restatement
(oracle/simple_np.py Domain.gradient_lsq) with the boundary values the solver set,
and exact for a linear field in the cells without boundary faces."""
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


@pytest.mark.parametrize("mesh", ["tet", "hex"])
def test_lsq_gradient_matches_oracle(mesh):
    m = mg.lid_cavity_tet(6, 6, 4, jitter=0.2, seed=5) if mesh == "tet" else mg.lid_cavity_hex(7)
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, m, mg.cavity_param("x", 2, mu=0.01))
        d = simple_np.SimpleNP(p).d
        a = np.array([1.5, -2.0, 0.75])
        U = 3.0 + d.g.cx @ a
        with NavierStokesSolver(p, {"gradient": 1}) as s:
            assert s.get_option("gradient") == 1
            s.set("U", U)
            s.CalculateVelocity()  # the gradients of U, V, W, P come first (BasicSolver.cpp:29 order)
            g = s.get("dUdX").reshape(-1, 3)
            BU = s.get("BU")
        ref = d.gradient_lsq(U, BU)
        scale = np.abs(ref).max()
        np.testing.assert_allclose(g, ref, rtol=0, atol=1e-12 * scale)
        interior = np.ones(d.nc, bool)
        interior[d.m.c1[d.m.bface]] = False
        assert interior.any()
        np.testing.assert_allclose(g[interior], np.broadcast_to(a, g[interior].shape), rtol=0, atol=1e-10)


def test_lsq_option_switches_back_and_rejects_bad_values():
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_hex(5), mg.cavity_param("x", 2, mu=0.01))
        with NavierStokesSolver(p, {}) as s:
            s.iterate(2)
            gg = s.get("dUdX")
            s.reset()
            s.set_option("gradient", 1)
            s.iterate(2)
            lsq = s.get("dUdX")
            s.reset()
            s.set_option("gradient", 0)
            s.iterate(2)
            assert np.array_equal(s.get("dUdX"), gg)
            assert not np.array_equal(lsq, gg)
            with pytest.raises(SysuError):
                s.set_option("gradient", 2)

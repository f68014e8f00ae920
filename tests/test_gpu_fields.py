"""Field transfers of the solver-level C ABI: every kind of field (cell, cell
gradient, face flux in reference face order, boundary record) survives a set/get
round trip, from pageable and from page-locked host memory, and the face order
matches the reference's (RUFace of the reference run)."""
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import _lib
from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300.solver import NavierStokesSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pinned", [False, True])
def test_field_round_trips(pinned):
    rng = np.random.default_rng(1)
    with tempfile.TemporaryDirectory() as d:
        p = mg.write_case(d, mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", 10, turb=True))
        with NavierStokesSolver(p) as s:
            s.iterate(2)
            for name in ("U", "P", "T", "dUdX", "dPdX", "RUFace", "BU", "BTem", "solid_T", "solid_dPhidX"):
                n = s.field_size(name)
                a = _lib.pinned_empty(n) if pinned else np.empty(n)
                a[:] = rng.standard_normal(n)
                s.set(name, a)
                out = _lib.pinned_empty(n) if pinned else None
                got = s.get(name, out=out)
                assert np.array_equal(got, a), name

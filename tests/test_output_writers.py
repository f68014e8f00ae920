"""Output writers (Tecplot FEBRICK files, tot.dat) against the reference's own output.

The reference binary (oracle/_ref/cycas_ref, the reference's src/*.cpp unmodified) runs
NSSolve on a small conjugate-heat-transfer k-epsilon channel and writes
tec/res####.dat and tot.dat (navier.cpp:13-97,243-337, HeatConductionSolver.cpp:330-361).
* CPU: the host writer (sysu_case_write_tecplot) fed with the reference's own final
  fields must reproduce its last Tecplot file byte for byte.
* GPU: nssolve with option "output" writes the same set of files; their structure
  (headers, zone lines, connectivity) matches exactly and the numbers to the 6
  printed digits, up to the last-digit rounding of values that differ by 1e-13.
"""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from sysu_cfd_heat_gb300 import _lib
from sysu_cfd_heat_gb300 import meshgen as mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "cycas_ref")
ENV = {"SYSU_ORACLE_GMRES_AS": "BiCGSTAB", "SYSU_ORACLE_SSOR_AS": "Jacobi", "SYSU_ORACLE_RTC": "1e-13"}
FIELDS = ["P", "U", "V", "W", "R", "T", "VisLam", "VisTur", "TE", "ED"]


def _case_rows(iters, noutput):
    rows = mg.cht_param("x", iters, turb=True)
    return [("output", noutput) if r[0] == "output" else r for r in rows]


def _run_reference(d):
    os.makedirs(os.path.join(d, "tec"), exist_ok=True)
    os.makedirs(os.path.join(d, "out"), exist_ok=True)
    subprocess.run([REF_BIN, "-paramfile", "param.in", "-nssolve", "-dump", "out", "-quiet"], cwd=d,
                   env=dict(os.environ, **ENV), check=True, capture_output=True, timeout=600)


def _tec_files(d):
    return sorted(f for f in os.listdir(os.path.join(d, "tec")) if f.startswith("res"))


@pytest.fixture(scope="module")
def ref_run():
    if not os.path.exists(REF_BIN):
        pytest.skip("oracle/_ref/cycas_ref not built (no reference sources installed)")
    d = tempfile.mkdtemp()
    mg.write_case(d, mg.cht_channel(8, 4, 2, 3), _case_rows(5, 2))
    _run_reference(d)
    yield d
    shutil.rmtree(d, ignore_errors=True)


def test_host_writer_reproduces_reference_bytes(ref_run):
    L = _lib.lib()
    L.sysu_case_write_tecplot.restype = C.c_int
    L.sysu_case_write_tecplot.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_char_p),
                                          C.POINTER(C.POINTER(C.c_double))]
    h = C.c_void_p()
    _lib.check(L.sysu_case_load(os.path.join(ref_run, "param.in").encode(), C.byref(h)))
    try:
        arrays = {f: np.fromfile(os.path.join(ref_run, "out", f + ".f64")) for f in FIELDS}
        arrays["solid_T"] = np.fromfile(os.path.join(ref_run, "out", "solid_T.f64"))
        names = list(arrays)
        cn = (C.c_char_p * len(names))(*[n.encode() for n in names])
        ca = (C.POINTER(C.c_double) * len(names))(*[arrays[n].ctypes.data_as(C.POINTER(C.c_double))
                                                    for n in names])
        out = os.path.join(ref_run, "ours.dat")
        _lib.check(L.sysu_case_write_tecplot(h, out.encode(), len(names), cn, ca))
    finally:
        L.sysu_case_free(h)
    last = _tec_files(ref_run)[-1]
    ref = open(os.path.join(ref_run, "tec", last), "rb").read()
    ours = open(out, "rb").read()
    assert ours == ref


def _tokens(path):
    with open(path) as f:
        return f.read().split()


@pytest.mark.gpu
def test_nssolve_output_files(ref_run):
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    with tempfile.TemporaryDirectory() as d:
        p = mg.write_case(d, mg.cht_channel(8, 4, 2, 3), _case_rows(5, 2))
        with NavierStokesSolver(p, {"rtc": 1e-13, "output": 1}) as s:
            s.NSSolve()
        assert _tec_files(d) == _tec_files(ref_run)
        for name in _tec_files(d):
            a, b = _tokens(os.path.join(d, "tec", name)), _tokens(os.path.join(ref_run, "tec", name))
            assert len(a) == len(b)
            for x, y in zip(a, b):
                if x == y:
                    continue
                fx, fy = float(x), float(y)  # only numbers may differ, in the last printed digit
                assert abs(fx - fy) <= 2e-5 * max(abs(fx), abs(fy)) + 1e-9, (name, x, y)
        a = open(os.path.join(d, "tot.dat")).read().splitlines()
        b = open(os.path.join(ref_run, "tot.dat")).read().splitlines()
        assert a[0] == b[0] and len(a) == len(b) == 2
        ta, tb = a[1].split(), b[1].split()
        assert ta[:2] == tb[:2]
        for x, y in zip(ta[2:], tb[2:]):
            assert abs(float(x) - float(y)) <= 1e-9 * max(abs(float(y)), 1.0)

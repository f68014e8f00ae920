"""CPU tests (no GPU): host-side case building vs the reference, the param.in
grammar and its quirks, and the C ABI's exported symbols."""
import ctypes
import os
import re
import tempfile

import numpy as np
import pytest

import make_golden
from sysu_cfd_heat_gb300 import meshgen as mg
from sysu_cfd_heat_gb300._lib import LIB_PATH, Case, SysuError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
CASES = make_golden.cases()

GEOM_F = ["cell_vol", "cell_x", "face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "bnd_distance"]
GEOM_I = ["cell_nface", "cell_rid", "cell_vert", "face_c1", "face_c2", "face_vert", "bnd_face", "bnd_rid"]


@pytest.mark.parametrize("name", ["cavity_hex6_tight", "cavity_tet_tight", "cht_ke_tight", "cavity_hex5_mlp"])
def test_geometry_bit_exact(name):
    """Faces, topology and CellFaceInfo geometry equal the reference's bit for bit."""
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    mesh, rows, _, _ = CASES[name]
    with tempfile.TemporaryDirectory() as tmp:
        c = Case(mg.write_case(tmp, mesh, rows))
        info = c.info()
        prefixes = [""] + (["solid_"] if info["has_solid"] else [])
        checked = 0
        for pre in prefixes:
            c2 = c.array(pre + "face_c2")
            inner = np.repeat(c2 >= 0, 3)
            for g in GEOM_F + GEOM_I:
                key = "geom_" + pre + g
                if key not in gold.files:
                    continue
                np.testing.assert_array_equal(c.array(pre + g), gold[key], err_msg=pre + g)
                checked += 1
            for g in ("face_xpac", "face_xnac"):
                a = np.where(inner, c.array(pre + g), 0.0)
                np.testing.assert_array_equal(a, gold["geom_" + pre + g], err_msg=pre + g)
            nbr = c.array(pre + "cell_nbr")
            r = gold["geom_" + pre + "cell_nbr"]
            m = r != -100
            np.testing.assert_array_equal(nbr[m], r[m])
        assert checked >= 14


def test_cht_interface_pairing():
    """Fluid and solid coupled faces are paired by enumeration order in the reference;
    the generated channel makes that order coincide with the shared geometric face."""
    mesh, rows, _, _ = CASES["cht_ke_tight"]
    with tempfile.TemporaryDirectory() as tmp:
        c = Case(mg.write_case(tmp, mesh, rows))
        i = c.info()
        fb = c.array("bnd_face")[i["NCoupledBnd"]:]
        sb = c.array("solid_bnd_face")[i["solid_NCoupledBnd"]:]
        fx = c.array("face_x").reshape(-1, 3)[fb]
        sx = c.array("solid_face_x").reshape(-1, 3)[sb]
        assert len(fb) == len(sb) > 0
        np.testing.assert_array_equal(fx, sx)


def _case_with_param(tmp, text: bytes):
    mg.write_msh(os.path.join(tmp, "mesh.msh"), mg.lid_cavity_hex(3))
    p = os.path.join(tmp, "param.in")
    with open(p, "wb") as f:
        f.write(text)
    return p


BASE = (b"gridfile, mesh.msh\r\nsteady, 11, 1e-6\r\nenergy, off\r\nrelaxation, 0.7, 0.3, 0.8\r\n"
        b"bound, 1, Hwall, 0.\r\nbound, 2, inlet, 1., 0., 0., 0., 1., 0.\r\n"
        b"volumn, 5, fluid, f, 0., 0., 0., 1., 0., 0.01, 0., 0.\r\n")


def test_param_crlf_blank_lines_and_comments_are_skipped():
    with tempfile.TemporaryDirectory() as tmp:
        Case(_case_with_param(tmp, b"// a comment\r\n\r\n" + BASE + b"\r\noutput, 5\r\n"))


def test_param_lf_blank_line_is_an_unknown_keyword():
    """readparamfile.cpp:27-28 skips only lines of length 1; an LF blank line is keyword ''."""
    with tempfile.TemporaryDirectory() as tmp:
        with pytest.raises(SysuError, match="no such command"):
            Case(_case_with_param(tmp, BASE.replace(b"\r\n", b"\n") + b"\n"))


def test_param_unknown_keyword_and_bad_values():
    with tempfile.TemporaryDirectory() as tmp:
        with pytest.raises(SysuError, match="no such command"):
            Case(_case_with_param(tmp, BASE + b"frobnicate, 1\r\n"))
    with tempfile.TemporaryDirectory() as tmp:
        with pytest.raises(SysuError, match="limiter"):
            Case(_case_with_param(tmp, BASE + b"limiter, superbee\r\n"))
    with tempfile.TemporaryDirectory() as tmp:
        with pytest.raises(SysuError, match="repeating bid"):
            Case(_case_with_param(tmp, BASE + b"bound, 2, outlet, 0.\r\n"))
    with tempfile.TemporaryDirectory() as tmp:
        with pytest.raises(SysuError, match="bid == 0"):
            Case(_case_with_param(tmp, BASE + b"bound, 0, sym\r\n"))


def test_missing_boundary_element_is_reported():
    """A mesh whose boundary elements do not cover every boundary face is rejected
    (the reference's CheckAndAllocate test, navier.cpp:497-503)."""
    m = mg.lid_cavity_hex(3)
    m.quads = m.quads[:-1]
    m.quad_ids = m.quad_ids[:-1]
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, m, mg.cavity_param("x", 2, mu=0.01))
        with pytest.raises(SysuError, match="boundary face"):
            Case(p)


def test_mesh_counts():
    with tempfile.TemporaryDirectory() as tmp:
        c = Case(mg.write_case(tmp, mg.lid_cavity_tet(4, 3, 2, jitter=0.2), mg.cavity_param("x", 2, mu=0.01)))
        i = c.info()
        assert i["Ncel"] == 4 * 3 * 2 * 6
        # every tet has 4 faces: 2F + B = 4 N
        F = i["Nfac"] - i["Nbnd"]
        assert 2 * F + i["Nbnd"] == 4 * i["Ncel"]
        assert np.all(c.array("cell_vol") > 0)
        np.testing.assert_allclose(c.array("cell_vol").sum(), 1.0, rtol=1e-13)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(LIB_PATH)
    names = set()
    inc = os.path.join(ROOT, "include")
    for h in os.listdir(inc):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(inc, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "while", "return", "sizeof", "defined"):
                names.add(m.group(1))
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


ALL_ARRAYS = GEOM_F + GEOM_I + ["face_xpac", "face_xnac", "cell_nbr", "cell_face", "face_bnd", "vert"]


def _load_all(param, threads):
    old = os.environ.get("SYSU_THREADS")
    os.environ["SYSU_THREADS"] = str(threads)
    try:
        c = Case(param)
        pre = [""] + (["solid_"] if c.info()["has_solid"] else [])
        return {p + g: c.array(p + g) for p in pre for g in ALL_ARRAYS}
    finally:
        if old is None:
            os.environ.pop("SYSU_THREADS")
        else:
            os.environ["SYSU_THREADS"] = old


@pytest.mark.parametrize("kind", ["tet", "cht"])
def test_threaded_preprocessing_is_identical(kind):
    """MSH read, face construction and geometry over threads give the same bytes
    as one thread (meshes above the threading thresholds: > 1 MB, > 20,000 cells)."""
    with tempfile.TemporaryDirectory() as tmp:
        if kind == "tet":
            p = mg.write_case(tmp, mg.lid_cavity_tet(20, 20, 20, jitter=0.2, seed=3), mg.cavity_param("x", 10, mu=0.01))
        else:
            p = mg.write_case(tmp, mg.cht_channel(48, 20, 6, 24), mg.cht_param("x", 10))
        assert os.path.getsize(os.path.join(tmp, "mesh.msh")) > (1 << 20)
        a = _load_all(p, 1)
        b = _load_all(p, 5)
        assert a.keys() == b.keys()
        for k in a:
            assert a[k].tobytes() == b[k].tobytes(), k


def test_threaded_reader_reports_the_reference_error():
    with tempfile.TemporaryDirectory() as tmp:
        p = mg.write_case(tmp, mg.lid_cavity_tet(20, 20, 20, jitter=0.2, seed=3), mg.cavity_param("x", 10, mu=0.01))
        msh = os.path.join(tmp, "mesh.msh")
        lines = open(msh).read().split("\n")
        k = len(lines) - 40  # an element near the end: a vertex that does not exist
        parts = lines[k].split()
        parts[-1] = str(10 ** 8)
        lines[k] = " ".join(parts)
        open(msh, "w").write("\n".join(lines))
        msgs = []
        for thr in (1, 5):
            os.environ["SYSU_THREADS"] = str(thr)
            try:
                with pytest.raises(SysuError) as e:
                    Case(p)
                msgs.append(e.value.msg)
            finally:
                os.environ.pop("SYSU_THREADS")
        assert msgs[0] == msgs[1] and "missing vertex" in msgs[0]

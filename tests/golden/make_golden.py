"""Generate the golden fixtures of tests/golden/ by running the compiled reference.

The reference binary (oracle/_ref/cycas_ref: the reference's own src/*.cpp, unmodified,
linked with the CPU LASPack restatement and the dump driver) runs each small seeded case
below and its outputs are stored as .npz:

* ``fields_*``  -- cell/face/boundary fields after N outer iterations;
* ``stage1_*``  -- iteration-1 intermediates (gradients, Apr, Rhie-Chow fluxes, p', ...);
* ``solve<k>_*`` -- the first linear systems (full CSR, b, x0, x) the reference solved;
* ``res``       -- Residual[0..3] and max per iteration.

Usage:  python tests/golden/make_golden.py   (needs oracle/_ref/cycas_ref; see oracle/Makefile)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sysu_cfd_heat_gb300 import meshgen as mg  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "cycas_ref")

# solver remap that the configs ask for: BiCGSTAB for the GMRES call sites, Jacobi for SSOR
REMAP = {"SYSU_ORACLE_GMRES_AS": "BiCGSTAB", "SYSU_ORACLE_SSOR_AS": "Jacobi"}


def cases():
    """name -> (mesh, param rows, iterations, env, solid_source)"""
    c = {}
    c["cavity_hex6_tight"] = (mg.lid_cavity_hex(6), mg.cavity_param("x", 20, mu=0.01), 20,
                              dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    c["cavity_tet_tight"] = (mg.lid_cavity_tet(5, 4, 3, jitter=0.2), mg.cavity_param("x", 15, mu=0.0025), 15,
                             dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    c["cavity_hex6_weno"] = (mg.lid_cavity_hex(6), mg.cavity_param("x", 10, mu=0.01, limiter="WENO"), 10,
                             dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    c["cavity_tet_barth"] = (mg.lid_cavity_tet(4, 4, 3, jitter=0.2), mg.cavity_param("x", 8, mu=0.0025, limiter="Barth"),
                             8, dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    c["cavity_hex5_mlp"] = (mg.lid_cavity_hex(5), mg.cavity_param("x", 8, mu=0.01, limiter="MLP"), 8,
                            dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    c["cht_ke_tight"] = (mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", 8, turb=True), 8,
                         dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    c["cht_lam_tight"] = (mg.cht_channel(8, 4, 2, 3), mg.cht_param("x", 8, turb=False), 8,
                          dict(REMAP, SYSU_ORACLE_RTC="1e-13"))
    # configuration 1 of the benchmark set: 24^3 lid cavity, Re 100, 300 iterations, 1e-8
    c["c1_cavity24"] = (mg.lid_cavity_hex(24), mg.cavity_param("x", 300, mu=0.01), 300,
                        dict(REMAP, SYSU_ORACLE_RTC="1e-8"))
    return c


FIELDS_CELL = ["U", "V", "W", "P", "T", "TE", "ED", "VisTur", "Apr"]
FIELDS_OTHER = ["RUFace", "BU", "BV", "BW", "BRo", "BTem", "BTE", "BED", "Bq"]
GEOM = ["cell_vol.f64", "cell_x.f64", "cell_nface.i32", "cell_face.i32", "cell_nbr.i32", "cell_rid.i32",
        "cell_vert.i32", "face_x.f64", "face_n.f64", "face_area.f64", "face_lambda.f64", "face_rlencos.f64",
        "face_xpac.f64", "face_xnac.f64", "face_c1.i32", "face_c2.i32", "face_bnd.i32", "face_vert.i32",
        "bnd_face.i32", "bnd_rid.i32", "bnd_distance.f64"]
STAGE1 = ["dUdX", "dVdX", "dWdX", "dPdX", "Apr", "Ustar", "Vstar", "Wstar", "RUFace_star", "dp", "dPdX_dp",
          "P1", "U1", "V1", "W1", "RUFace1"]


def run_case(name, mesh, rows, iters, env, out_dir, dump_solves=4, keep_all=True):
    with tempfile.TemporaryDirectory() as tmp:
        mg.write_case(tmp, mesh, rows)
        for sub in ("out", "s1", "solves"):
            os.makedirs(os.path.join(tmp, sub))
        e = dict(os.environ)
        e.update(env)
        e["SYSU_ORACLE_DUMP_DIR"] = os.path.join(tmp, "solves")
        e["SYSU_ORACLE_DUMP_MAX"] = str(dump_solves)
        cmd = [REF_BIN, "-paramfile", "param.in", "-iters", str(iters), "-dump", "out", "-stage1", "s1", "-quiet"]
        if keep_all:
            cmd.append("-geom")
        subprocess.run(cmd, cwd=tmp, env=e, check=True, capture_output=True)
        data = {}
        meta = {}
        for line in open(os.path.join(tmp, "out", "meta.txt")):
            k, v = line.split()
            meta[k] = int(v)
        data["meta_keys"] = np.array(list(meta.keys()))
        data["meta_vals"] = np.array(list(meta.values()), dtype=np.int64)
        res = np.loadtxt(os.path.join(tmp, "out", "iters.txt"), ndmin=2)
        data["res"] = res
        names = FIELDS_CELL + FIELDS_OTHER + ["dPhidX", "dPdX"]
        if meta.get("Solve3DHeatConduction"):
            names += ["solid_T", "solid_BTem", "solid_Bq", "solid_dPhidX"]
        if iters >= 100:
            names = ["U", "V", "W", "P", "RUFace"]
        for f in names:
            p = os.path.join(tmp, "out", f + ".f64")
            if os.path.exists(p):
                data["fields_" + f] = np.fromfile(p, dtype=np.float64)
        if keep_all:
            for pre in ("", "solid_"):
                for g in GEOM:
                    p = os.path.join(tmp, "out", pre + g)
                    if os.path.exists(p):
                        dt = np.int32 if g.endswith(".i32") else np.float64
                        data["geom_" + pre + g.split(".")[0]] = np.fromfile(p, dtype=dt)
            for f in STAGE1:
                p = os.path.join(tmp, "s1", f + ".f64")
                if os.path.exists(p):
                    data["stage1_" + f] = np.fromfile(p, dtype=np.float64)
            sol = os.path.join(tmp, "solves")
            man = os.path.join(sol, "solves.txt")
            if os.path.exists(man):
                for line in open(man):
                    parts = line.split()
                    k = int(parts[0])
                    pre = f"solve{k}_"
                    data[pre + "method"] = np.array(parts[1])
                    data[pre + "precond"] = np.array(parts[2])
                    data[pre + "eps"] = np.array(float(parts[5]))
                    data[pre + "maxit"] = np.array(int(parts[6]))
                    data[pre + "omega"] = np.array(float(parts[7]))
                    data[pre + "iters"] = np.array(int(parts[8]))
                    data[pre + "acc"] = np.array(float(parts[9]))
                    for tag, dt in (("rowptr.i32", np.int32), ("col.i32", np.int32), ("val.f64", np.float64),
                                    ("b.f64", np.float64), ("x0.f64", np.float64), ("x.f64", np.float64)):
                        data[pre + tag.split(".")[0]] = np.fromfile(os.path.join(sol, f"solve_{k:04d}_{tag}"), dtype=dt)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **data)
        return data


def main():
    if not os.path.exists(REF_BIN):
        sys.exit(f"{REF_BIN} missing: build it with make -C oracle")
    for name, (mesh, rows, iters, env) in cases().items():
        keep = not name.startswith("c1_")
        d = run_case(name, mesh, rows, iters, env, HERE, keep_all=keep)
        print(name, "iterations", len(d["res"]), "final max residual", d["res"][-1, -1])


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Benchmark of the SIMPLE hot path: outer iterations per second on the 2M-cell case.

Workload (the configuration the headline metric is quoted on): unit-cube lid-driven
cavity at Re = 400 on 80 x 80 x 52 hexes cut into 6 tets each (1,996,800 cells),
interior nodes jittered by U(-0.2h, 0.2h) from seed 20261203; rho = 1, mu = 0.0025,
lid u = 1; under-relaxation 0.7 (u, v, w) / 0.3 (p); BiCGSTAB + Jacobi for momentum,
Jacobi-CG for p', relative tolerance 1e-8 for every solve; plain FP64.  Synthetic
input: the reference publishes no mesh or benchmark data.

One step = one SIMPLE outer iteration (momentum assembly + 3-RHS solve, Rhie-Chow,
p' assembly + CG solve, corrections) with the fields resident in HBM.  The timed
iterations start from the initial state (the solver is reset after warm-up), so they
are the same iterations the CPU sample times.  ``e2e`` runs the same iterations
through the C ABI with host buffers: every step uploads U, V, W, P and the face
fluxes from host memory and reads U, V, W, P back.

``--impl reference`` times the reference's own CPU code (oracle/_ref/cycas_ref_o3: the
reference's src/*.cpp + the LASPack restatement at -O3 -march=native) on the same case,
single-threaded as the reference is and pinned to one core, for the same --steps outer
iterations (stopping early only past --ref-budget seconds).

With torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path has no data-parallel exchange); value = total iterations / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SIMPLE iters/s @2M cells; p' solve time to 1e-8: learned+FP32 vs plain FP64"
WORKLOADS = {
    # name: (nx, ny, nz)
    "c3": (80, 80, 52),
    "small": (20, 20, 13),
}
RE_MU = 0.0025
SEED = 20261203
RTC = 1e-8
L2_BYTES = 129 * 1024 * 1024
FP64_PEAK_TFLOPS = 1.25
LEARN_ITERS = 10   # outer iterations that train the learned preconditioner
LEARN_STEPS = 64   # Adam steps per training outer iteration
LEARN_C5_ITERS = 40  # training outer iterations of the --learned-c5 run
LEARN_C5_MG = 10     # training outer iterations of its learned multigrid form


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", str(r)))
    return r, w, lr


def case_dir(workload: str) -> str:
    from sysu_cfd_heat_gb300 import meshgen as mg

    nx, ny, nz = WORKLOADS[workload]
    d = os.path.join(tempfile.gettempdir(), f"sysu_bench_{workload}_{nx}x{ny}x{nz}_s{SEED}")
    p = os.path.join(d, "param.in")
    if not os.path.exists(p):
        tmp = d + ".tmp%d" % os.getpid()
        mesh = mg.lid_cavity_tet(nx, ny, nz, jitter=0.2, seed=SEED)
        mg.write_case(tmp, mesh, mg.cavity_param("x", 100000, mu=RE_MU, urf=(0.7, 0.3, 0.8)))
        try:
            os.rename(tmp, d)
        except OSError:
            pass
    return p


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cg_bytes_per_iter(n: int, nnz: int, fp32: bool = False) -> float:
    """Algorithmic bytes of one CG iteration of the p' kernel (two phases):
    S reads the matrix once (values + int32 columns), gathers z once (one value per
    row), reads and writes p and q; X reads p, q, x (or the correction e), r,
    D^-1 and writes x (e), r, z.  FP64: nnz*12 + 104*N; FP32 recurrences:
    nnz*8 + 52*N."""
    if fp32:
        return nnz * 8 + 52 * n
    return nnz * 12 + 104 * n


def cg_flops_per_iter(n: int, nnz_true: int) -> float:
    """FP64 flops of one CG iteration: 2 per stored-true matrix entry, 6 per row in S
    (p, q updates, p.q), 7 per row in X (x, r, z, r.z; r.r, which only serves the
    stopping test, is estimated in FP32 and taken exactly only near the threshold)."""
    return 2.0 * nnz_true + 13.0 * n


def host_cpu() -> dict:
    """Host cores and CPU model of this machine (the CPU baseline's record)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None and os.path.exists("/proc/cpuinfo"):
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    return {"nproc": os.cpu_count(), "cpu_model": model or "unknown"}


def cpu_reference_run(param: str, iters: int, budget_s: float, timeout_s: float, build: str = "o3",
                      env_extra: dict | None = None):
    """Run the reference binary on the case, single-threaded and pinned to one core
    (the last core this process may use); stops after `iters` outer iterations or
    once they add up to more than budget_s.  build: "o3" (-O3 -march=native, the
    primary CPU baseline), "o2" (the parity build) or "g" (the reference's shipped
    flags, -g without optimisation).  Returns (per-iteration seconds, setup s,
    error or None, record)."""
    exe = os.path.join(ROOT, "oracle", "_ref", {"o3": "cycas_ref_o3", "o2": "cycas_ref", "g": "cycas_ref_g"}[build])
    if not os.path.exists(exe):
        return None, None, f"oracle/_ref/{os.path.basename(exe)} not built (no reference sources on this machine)", {}
    d = os.path.dirname(param)
    env = dict(os.environ, SYSU_ORACLE_GMRES_AS="BiCGSTAB", SYSU_ORACLE_SSOR_AS="Jacobi", SYSU_ORACLE_RTC=str(RTC))
    env.update(env_extra or {})
    try:
        core = max(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        core = None
    rec = dict(host_cpu(), binary="oracle/_ref/" + os.path.basename(exe), pinned_core=core,
               flags={"o3": "-O3 -march=native", "o2": "-O2", "g": "-g (the reference makefile's flags)"}[build])

    def pin():
        if core is not None:
            os.sched_setaffinity(0, {core})

    with tempfile.TemporaryDirectory() as tmp:
        tfile = os.path.join(tmp, "timing.txt")
        cmd = [exe, "-paramfile", os.path.basename(param), "-iters", str(iters), "-quiet", "-timing", tfile]
        t0 = time.time()
        p = subprocess.Popen(cmd, cwd=d, env=env, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                             preexec_fn=pin)
        setup, its = None, []
        while p.poll() is None:
            time.sleep(0.5)
            setup, its = _read_timing(tfile)
            el = time.time() - t0
            if el > timeout_s or (its and sum(its) > budget_s):
                p.kill()
                p.wait()
                break
        setup, its = _read_timing(tfile)
        return its, setup, None, rec


def cpu_rate(its):
    """(iterations/s, description): the mean over outer iterations 2.. when more
    than one finished, else iteration 1."""
    if len(its) >= 2:
        return (len(its) - 1) / sum(its[1:]), f"mean over outer iterations 2..{len(its)}"
    return 1.0 / its[0], "outer iteration 1"


def _read_timing(path):
    setup, its = None, []
    if not os.path.exists(path):
        return setup, its
    for line in open(path):
        parts = line.split()
        if not parts:
            continue
        if parts[0] == "setup_s":
            setup = float(parts[1])
        elif parts[0] == "iter" and "total_s" in parts:
            its.append(float(parts[parts.index("total_s") + 1]))
    return setup, its


def run_reference(args, r, w):
    if r != 0:
        return
    param = case_dir(args.workload)
    nx, ny, nz = WORKLOADS[args.workload]
    its, setup, err, rec = cpu_reference_run(param, max(1, args.steps), args.ref_budget, args.ref_budget + 600)
    base = {"impl": "reference", "metric": METRIC, "unit": "iters/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_of(args)}
    if err or not its:
        base["unavailable"] = err or "the reference completed no outer iteration within the time budget"
        print(json.dumps(base))
        return
    tot = sum(its)
    v = len(its) / tot
    sample = (f"outer iterations 1..{len(its)} of the {args.workload} case ({6 * nx * ny * nz} cells), "
              f"set-up ({setup:.1f} s) excluded, {rec['flags']}, 1 thread pinned to core {rec['pinned_core']}")
    base.update({"value": v, "ms_per_step": 1000 * tot / len(its), "steps": len(its),
                 "cpu_baseline": {"value": v, "unit": "iters/s", "cores": 1, "kind": "reference", "sample": sample,
                                  "host": rec},
                 "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    print(json.dumps(base))


def spmv_bytes(n: int, nnz: int, sv: int) -> float:
    """Algorithmic bytes of one y = A x: nnz (value + int32 column), N+1 row pointers,
    x and y once each."""
    return nnz * (sv + 4) + 4 * (n + 1) + 2 * n * sv


def spmv_sweep(s, n: int, nnz: int, hbm: float, at=(1, 10, 100), reps: int = 10) -> dict:
    """y = A x on the p' and momentum matrices as assembled after the given outer
    iterations (FP64 values and their FP32 copy), L2 flushed before each product,
    by four kernel forms: one row per thread over a full grid (the top-level
    figures), the persistent bulk-copy ring (`ring`), the per-warp cp.async
    pipeline (`async`) and x staged in shared memory per block (`staged_x`); and
    the first and last of those in steady state (`steady`, `staged_x_steady`:
    products back to back alternating between two full copies of the operands,
    more than the L2 holds, as the products of an iterative solve run)."""
    out = {}
    s.reset()
    done = 0
    for k in at:
        s.iterate(k - done)
        done = k
        row = {}
        for which in ("p", "mom"):
            for fp32 in (False, True):
                b = spmv_bytes(n, nnz, 4 if fp32 else 8)
                res = {}
                for name, variant in (("stream", 0), ("ring", 100), ("async", 200), ("staged_x", 300)):
                    s.set_option("spmv_variant", variant)
                    ms = s.spmv_timing(which, fp32, reps)
                    gbs = b / (ms / 1000.0) / 1e9
                    res[name] = {"ms": ms, "GB/s": gbs, "frac_of_hbm": gbs / hbm}
                for name, variant in (("stream", 0), ("staged_x", 300)):
                    s.set_option("spmv_variant", variant)
                    ms = s.spmv_timing(which, fp32, reps, steady=True)
                    gbs = b / (ms / 1000.0) / 1e9
                    res[name + "_steady"] = {"ms": ms, "GB/s": gbs, "frac_of_hbm": gbs / hbm}
                s.set_option("spmv_variant", 0)
                entry = dict(res["stream"])
                entry["algorithmic_bytes"] = b
                entry["ring"] = res["ring"]
                entry["async"] = res["async"]
                entry["staged_x"] = res["staged_x"]
                entry["steady"] = res["stream_steady"]
                entry["staged_x_steady"] = res["staged_x_steady"]
                row[f"{which}_{'fp32' if fp32 else 'fp64'}"] = entry
        out[f"after_outer_iteration_{k}"] = row
    return out


def config_of(args):
    nx, ny, nz = WORKLOADS[args.workload]
    return {"workload": f"lid-driven cavity Re 400, {nx}x{ny}x{nz} hexes x 6 jittered tets "
                        f"({6 * nx * ny * nz} cells), seed {SEED}",
            "cells": 6 * nx * ny * nz, "solvers": "momentum 3-RHS BiCGSTAB+Jacobi, p' Jacobi-CG, rtol 1e-8",
            "precision": "fp64",
            "l2": ("inputs larger than L2 (mesh, fields and matrices > 129 MB)" if nx * ny * nz * 6 > 1000000
                   else "small case: resident in L2 (development runs only)"),
            "parallelism": "replicas"}


def batch_case_dirs():
    """The 48 lid-driven hex cavities of the batch form (edge 12..64 cells, Re 50..1000)."""
    from sysu_cfd_heat_gb300 import meshgen as mg

    out = []
    for k, (L, re) in enumerate(mg.batch_cavities()):
        d = os.path.join(tempfile.gettempdir(), f"sysu_bench_batch_s{SEED}_{k}_{L}")
        p = os.path.join(d, "param.in")
        if not os.path.exists(p):
            tmp = d + ".tmp%d" % os.getpid()
            mg.write_case(tmp, mg.lid_cavity_hex(L), mg.cavity_param("x", 100000, mu=1.0 / re))
            try:
                os.rename(tmp, d)
            except OSError:
                pass
        out.append((p, L, re))
    return out


def batch_form(args):
    """48 independent cavities advanced together: one CUDA graph replay = one outer
    iteration of every case (each case on its own graph branch), p' in FP32 CG with
    FP64 reliable updates, each case's persistent-solver grid (SMs, i.e. rows per
    warp) chosen by the autotuner; against the same cases run one after another
    with ordinary launches and full-GPU grids."""
    from sysu_cfd_heat_gb300.batch import CaseBatch, DEFAULT_CAPS

    t0 = time.perf_counter()
    cases = batch_case_dirs()
    gen_s = time.perf_counter() - t0
    cells = sum(L ** 3 for _, L, _ in cases)
    with CaseBatch([p for p, _, _ in cases], {"rtc": RTC, "p.mixed": 1}) as b:
        t0 = time.perf_counter()
        tune = b.tune(DEFAULT_CAPS)
        tune_s = time.perf_counter() - t0
        b.capture()
        b.replay(args.warmup)
        for c in b.cases:
            c.reset()
        ms = b.replay(args.steps)
        b.check()
        u64 = [c.get("U") for c in b.cases]
        # the whole loop in FP32 with FP64 refinement: momentum too (u, v, w each by
        # BiCGSTAB with FP32 inner iterations in FP64 defect correction), same caps
        for c in b.cases:
            c.set_option("mom.mixed", 1)
            c.reset()
        b.capture()
        b.replay(args.warmup)
        for c in b.cases:
            c.reset()
        ms_m = b.replay(args.steps)
        b.check()
        err_m = max(float(np.linalg.norm(c.get("U") - u) / max(np.linalg.norm(u), 1e-300)) for c, u in zip(b.cases, u64))
        # p' by the multigrid flexible CG as well (each case's hierarchy built in the
        # capture's eager iteration; both solves loop on the device inside the graph)
        for c in b.cases:
            c.set_option("p.mixed", 0)
            c.set_option("p.precond", 4)
            c.reset()
        b.capture()
        b.replay(args.warmup)
        for c in b.cases:
            c.reset()
        ms_g = b.replay(args.steps)
        b.check()
        err_g = max(float(np.linalg.norm(c.get("U") - u) / max(np.linalg.norm(u), 1e-300)) for c, u in zip(b.cases, u64))
        for c in b.cases:
            c.set_option("p.precond", 1)
            c.set_option("p.mixed", 1)
            c.set_option("mom.mixed", 0)
        b.set_caps([0] * len(cases))
        for c in b.cases:
            c.reset()
        b.run_sequential(1)
        for c in b.cases:
            c.reset()
        seq_ms = b.run_sequential(args.steps)
    return {"cases": len(cases), "cells_total": cells, "edge_cells": [L for _, L, _ in cases],
            "reynolds": [round(re, 1) for _, _, re in cases],
            "batch_iters_per_s": args.steps / (ms / 1000.0),
            "case_iters_per_s": len(cases) * args.steps / (ms / 1000.0),
            "cell_iters_per_s": cells * args.steps / (ms / 1000.0),
            "ms_per_batch_iteration": ms / args.steps,
            "sequential_ms_per_batch_iteration": seq_ms / args.steps,
            "speedup_vs_sequential": seq_ms / ms if ms > 0 else None,
            "precision": "momentum BiCGSTAB FP64, p' CG FP32 recurrences + FP64 reliable updates, eps 1e-8",
            "fp32_momentum_too": {"ms_per_batch_iteration": ms_m / args.steps,
                                  "speedup_vs_sequential": seq_ms / ms_m if ms_m > 0 else None,
                                  "precision": "momentum u, v, w by one BiCGSTAB with FP32 recurrences + FP64 "
                                               "residual replacement (its loop a WHILE node of the graph), p' as above",
                                  "U_rel_l2_vs_fp64_momentum_max_over_cases": err_m},
            "multigrid_pressure_too": {"ms_per_batch_iteration": ms_g / args.steps,
                                       "speedup_vs_sequential": seq_ms / ms_g if ms_g > 0 else None,
                                       "precision": "momentum as fp32_momentum_too, p' by flexible CG (FP32 "
                                                    "recurrences + FP64 reliable updates) with the aggregation-"
                                                    "multigrid cycle, its loop a WHILE node of the graph",
                                       "U_rel_l2_vs_fp64_momentum_max_over_cases": err_g},
            "autotuner": {"candidates_sms": list(DEFAULT_CAPS), "sm_cap": tune["sm_cap"],
                          "measured_makespan_ms": tune["measured_makespan_ms"], "seconds": tune_s},
            "mesh_generation_seconds": gen_s}


def c2_case_dir():
    """Configuration 2: k-epsilon conjugate-heat-transfer channel, fluid 160 x 40 x 40 hexes
    (2.0 x 0.5 x 0.5 m) bonded to a 160 x 8 x 40 solid slab (0.1 m), u_in = 1 m/s, 5 % inlet
    turbulence with a 0.05 m mixing length, nu = 1e-5, k_s = 15 W/m/K."""
    from sysu_cfd_heat_gb300 import meshgen as mg

    d = os.path.join(tempfile.gettempdir(), "sysu_bench_c2_160x40x40")
    p = os.path.join(d, "param.in")
    if not os.path.exists(p):
        tmp = d + ".tmp%d" % os.getpid()
        mg.write_case(tmp, mg.cht_channel(160, 40, 8, 40), mg.cht_param("x", 100000, nu=1e-5, k_solid=15.0))
        try:
            os.rename(tmp, d)
        except OSError:
            pass
    return p


def c2_form(args):
    """Configuration 2 on the GPU (k-epsilon CHT channel, 256,000 + 51,200 cells, volumetric
    source 1e6 W/m^3 in the solid): outer iterations/s of the sequential form (the
    reference's order, FP64), of the batched scalar form (u, v, w as one 3-RHS BiCGSTAB;
    k, eps and T as one three-matrix launch), of the mixed-precision form (p' by the
    Jacobi-CG with FP32 recurrences; momentum, k, eps, T and the solid T with FP32
    iterations and FP64 residuals) and of the multigrid form (the same with p' by the
    multigrid flexible CG), all from the initial state, p' at the reference's
    1000-iteration cap; the last outer iteration's p' iterations and status, and the
    mixed forms' fields after the steps against the sequential form's (relative L2)."""
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    p = c2_case_dir()
    out = {}
    steps = max(args.steps, 10)
    with NavierStokesSolver(p, {"rtc": RTC, "solid_source": 1e6}) as s:
        info = s.info()
        fields = ("U", "V", "W", "P", "T", "TE", "ED", "solid_T")
        ref = {}
        mixed = {"scalars_batched": 0, "ke.mixed": 1, "t.mixed": 1, "ts.mixed": 1, "mom.mixed": 1}
        forms = (("sequential_fp64", {"scalars_batched": 0}), ("batched_scalars_fp64", {"scalars_batched": 1}),
                 ("mixed_fp32_fp64", dict(mixed, **{"p.mixed": 1, "p.precond": 1})),
                 ("multigrid_fp32_fp64", dict(mixed, **{"p.mixed": 0, "p.precond": 4})))
        for name, opts in forms:
            for k, v in opts.items():
                s.set_option(k, v)
            s.reset()
            s.iterate(args.warmup)
            s.reset()
            s.timer_start()
            done = s.iterate(steps)
            ms = s.timer_stop()
            st = s.solve_stats()
            out[name] = {"iters_per_s": done / (ms / 1000.0), "ms_per_step": ms / done,
                         "k_eps_T_iters_last": [st["k"]["iters"][0], st["eps"]["iters"][0], st["T"]["iters"][0]],
                         "p_iters_last": st["p"]["iters"][0], "p_status_last": st["p"]["status"][0],
                         "max_residual_after": float(max(s.Residual))}
            if name == "sequential_fp64":
                ref = {f: s.get(f) for f in fields}
            elif name in ("mixed_fp32_fp64", "multigrid_fp32_fp64"):
                out[name]["field_rel_l2_vs_fp64"] = max(
                    float(np.linalg.norm(s.get(f) - ref[f]) / max(np.linalg.norm(ref[f]), 1e-300)) for f in fields)
        for k in ("p.mixed", "ke.mixed", "t.mixed", "ts.mixed", "mom.mixed"):
            s.set_option(k, 0)
        s.set_option("p.precond", 1)
        out["cells"] = {"fluid": info["Ncel"], "solid": info["solid_Ncel"]}
        out["steps"] = steps
    return out


def c5_learned_run(args):
    """Configuration 5 (not part of the default run: --learned-c5): configuration 2 scaled
    up, fluid 320 x 80 x 160 hexes (4,096,000 cells) + solid 320 x 16 x 160 (819,200).
    The learned p' form trains during the first LEARN_C5_ITERS outer iterations, then the
    p' system of the next outer iteration is solved to 1e-8 by flexible CG with the
    network and, from the same state, by plain FP64 Jacobi-CG, the mixed FP32 CG, the
    multigrid flexible CG and the multigrid flexible CG with the network as its
    post-smoother (trained from that state for LEARN_C5_MG outer iterations); each
    method's fields after that outer iteration against the FP64 CG's."""
    from sysu_cfd_heat_gb300 import meshgen as mg
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    d = os.path.join(tempfile.gettempdir(), "sysu_bench_c5_320x80x160")
    p = os.path.join(d, "param.in")
    t0 = time.perf_counter()
    if not os.path.exists(p):
        tmp = d + ".tmp%d" % os.getpid()
        mg.write_case(tmp, mg.cht_channel(320, 80, 16, 160), mg.cht_param("x", 100000, nu=1e-5, k_solid=15.0))
        os.rename(tmp, d)
    gen_s = time.perf_counter() - t0
    out = {"mesh_generation_s": gen_s}
    with NavierStokesSolver(p, {"rtc": RTC, "solid_source": 1e6, "timing": 1, "p.maxit": 100000}) as s:
        info = s.info()
        out["cells"] = {"fluid": info["Ncel"], "solid": info["solid_Ncel"]}
        s.set_option("p.learned", 1)
        s.set_option("p.learn_iters", LEARN_C5_ITERS)
        s.set_option("p.learn_steps", LEARN_STEPS)
        t0 = time.perf_counter()
        s.iterate(LEARN_C5_ITERS)
        s.sync()
        out["training_s"] = time.perf_counter() - t0
        state = {f: s.get(f) for f in ("U", "V", "W", "P", "RUFace", "TE", "ED", "VisTur", "T", "solid_T")}
        res, fields = {}, {}
        forms = (("fp64_cg", {"p.learned": 0, "p.mixed": 0, "p.precond": 1}),
                 ("mixed_cg", {"p.learned": 0, "p.mixed": 1, "p.precond": 1}),
                 ("multigrid_fcg", {"p.learned": 0, "p.mixed": 0, "p.precond": 4}),
                 ("learned_fcg", {"p.learned": 1, "p.mixed": 0, "p.precond": 1}),
                 ("learned_multigrid_fcg", {"p.learned": 1, "p.mixed": 0, "p.precond": 4}))
        for name, opts in forms:
            if name == "learned_multigrid_fcg":
                # train the post-smoother from the same state: LEARN_C5_MG outer iterations
                for k, v in opts.items():
                    s.set_option(k, v)
                s.set_option("p.learn_reset", 1)
                s.set_option("p.learn_iters", LEARN_C5_MG)
                for f, a in state.items():
                    s.set(f, a)
                t0 = time.perf_counter()
                s.iterate(LEARN_C5_MG)
                s.sync()
                out["training_multigrid_s"] = time.perf_counter() - t0
            for k, v in opts.items():
                s.set_option(k, v)
            if name == "multigrid_fcg":
                # hierarchy set-up and graph capture at the first multigrid solve (the
                # learned multigrid form's happen in its training): not timed
                for f, a in state.items():
                    s.set(f, a)
                s.CalculateVelocity()
                s.CalculatePressure()
            for f, a in state.items():
                s.set(f, a)
            s.CalculateVelocity()
            s.CalculatePressure()
            s.check()
            st = s.solve_stats()["p"]
            res[name] = {"ms": s.timing()[0], "iters": st["iters"][0], "rel_residual": st["res"][0],
                         "converged": st["status"][0] == 0}
            fields[name] = {f: s.get(f) for f in ("U", "V", "W", "P")}
        for name in res:
            res[name]["field_rel_l2_vs_fp64_cg"] = max(
                float(np.linalg.norm(fields[name][f] - fields["fp64_cg"][f]) /
                      max(np.linalg.norm(fields["fp64_cg"][f]), 1e-300)) for f in fields[name])
        out["p_solve_to_1e-8_after_training"] = res
        out["training_outer_iterations"] = LEARN_C5_ITERS
    return out


# The forms of the p' solve timed side by side at a matched residual: every form
# starts from the same initial state and runs the same outer iterations with p'
# solved to the 1e-8 relative residual (no iteration cap).
# every form but the first runs its Krylov solves with FP32 recurrences: p' as
# named, momentum (u, v, w together) by BiCGSTAB with FP64 residual replacement
MOM32 = {"mom.mixed": 1}
MOM32_TEXT = "; momentum u, v, w by one BiCGSTAB with FP32 recurrences + FP64 residual replacement"
P_FORMS = (
    ("fp64", {}, "Jacobi-CG, FP64 (the drop-in's method without the reference's 1000-iteration cap); "
                 "momentum by the FP64 3-RHS BiCGSTAB"),
    ("mixed_fp32_fp64", {"p.mixed": 1, **MOM32}, "Jacobi-CG, FP32 recurrences + FP64 reliable updates" + MOM32_TEXT),
    ("multigrid_fp32_fp64", {"p.precond": 4, **MOM32},
     "flexible CG, FP32 recurrences + FP64 reliable updates, aggregation-multigrid V-cycle" + MOM32_TEXT),
    ("learned_multigrid_fp32_fp64", {"p.precond": 4, "p.learned": 1, "p.learn_level": 2, **MOM32},
     "as multigrid_fp32_fp64 with the trained message-passing network as the post-smoother of the cycle's "
     "second coarse level"),
    ("learned_multigrid_level1_fp32_fp64", {"p.precond": 4, "p.learned": 1, "p.learn_level": 1, **MOM32},
     "the same with the network on the first coarse level"),
    ("learned_multigrid_level0_fp32_fp64", {"p.precond": 4, "p.learned": 1, "p.learn_level": 0, **MOM32},
     "the same with the network as the finest level's post-smoother"),
    ("learned_network_fp32_fp64", {"p.learned": 1, **MOM32},
     "flexible CG, FP32 recurrences + FP64 reliable updates, the trained network as the whole preconditioner"
     + MOM32_TEXT),
)
P_OPTION_DEFAULTS = {"p.mixed": 0, "p.learned": 0, "p.precond": 1, "p.learn_level": 2, "mom.mixed": 0}


def pair_text(opts) -> str:
    """How a learned form's training pairs are made."""
    if not opts.get("p.precond"):
        return "(b, x*) and (b - A x1, x* - x1) per p' solve, x1 = solve to 1e-2"
    if opts.get("p.learn_level", 2) == 0:
        return ("(b, x*) and (b - A x1, x* - x1) per p' solve, x1 = solve to 1e-2, as post-smoother pairs "
                "(r - A z2, e - z2) of the finest level")
    return ("per p' solve, the right-hand sides r_l the cycle hands the network's level for the finest residuals "
            "b and b - A x1 (x1 = solve to 1e-2), their solutions e_l on that level (flexible CG with the "
            "hierarchy below it, to 1e-6), as post-smoother pairs (r_l - A_l z_l, e_l - z_l) of that level")


def matched_forms(s, args, n, nnz, hbm):
    """Outer iterations/s of every p' form at a matched 1e-8 residual, the p' solve
    time and iterations, and the fields' relative L2 difference from the FP64
    form's after the same iterations.  The learned forms first train during
    LEARN_ITERS outer iterations (plain solves generating the pairs, LEARN_STEPS
    Adam steps each); the fields are then reset and the same iterations timed
    with the trained network (training is not in the timed region)."""
    s.set_option("p.maxit", 100000)
    out, ref = {}, None
    for name, opts, what in P_FORMS:
        for k, v in P_OPTION_DEFAULTS.items():
            s.set_option(k, v)
        for k, v in opts.items():
            s.set_option(k, v)
        entry = {"method": what}
        if opts.get("p.learned"):
            s.set_option("p.learn_reset", 1)
            s.set_option("p.learn_iters", LEARN_ITERS)
            s.set_option("p.learn_steps", LEARN_STEPS)
            s.reset()
            t0 = time.perf_counter()
            s.iterate(LEARN_ITERS)
            s.sync()
            entry["training"] = {"outer_iterations": LEARN_ITERS, "adam_steps_per_iteration": LEARN_STEPS,
                                 "seconds_incl_plain_solves": time.perf_counter() - t0,
                                 "pairs": pair_text(opts),
                                 "loss": "residual norm ||A(z - e)||^2 / ||A e||^2"}
        else:
            s.reset()
            s.iterate(1)  # warm-up: hierarchy set-up, graph capture
        s.reset()
        tot, pm, mm, pit = 0.0, [], [], []
        for k in range(args.steps):
            s.timer_start()
            s.iterate(1)
            tot += s.timer_stop()
            pm.append(s.timing()[0])
            mm.append(s.timing()[1])
            st = s.solve_stats()["p"]
            pit.append(st["iters"][0])
            if st["status"][0] != 0:
                entry["p_status_not_converged"] = st["status"][0]
        fields = {f: s.get(f) for f in ("U", "V", "W", "P")}
        if ref is None:
            ref = fields
        entry.update({"iters_per_s": args.steps / (tot / 1000.0), "ms_per_step": tot / args.steps,
                      "p_solve_ms_mean": statistics.mean(pm), "p_iters_mean": statistics.mean(pit),
                      "mom_solve_ms_mean": statistics.mean(mm),
                      "field_rel_l2_vs_fp64": max(float(np.linalg.norm(fields[f] - ref[f]) /
                                                        max(np.linalg.norm(ref[f]), 1e-300)) for f in fields)})
        if name == "mixed_fp32_fp64":
            b32 = cg_bytes_per_iter(n, nnz, fp32=True)
            init32 = nnz * 12 + 40 * n
            ach32 = statistics.mean([(it * b32 + init32) / (ms / 1000.0) / 1e9 for it, ms in zip(pit, pm) if ms > 0])
            entry["roofline"] = {"bound": "hbm", "kernel": "k_cg_mixed_pipe", "achieved": ach32, "peak": hbm,
                                 "unit": "GB/s", "frac": ach32 / hbm, "algorithmic_bytes_per_cg_iteration": b32}
        out[name] = entry
    for k, v in P_OPTION_DEFAULTS.items():
        s.set_option(k, v)
    s.set_option("p.maxit", 1000)
    base = out["fp64"]["iters_per_s"]
    for name in out:
        out[name]["speedup_vs_fp64"] = out[name]["iters_per_s"] / base
    out["steps"] = args.steps
    out["p_eps"] = RTC
    out["target"] = ("learned + mixed-precision form at >= 3x the FP64 form's outer iterations/s, fields within "
                     "1e-6 relative L2")
    return out


def cpu_survey(args) -> dict:
    """--cpu-survey (not part of the default run; minutes of CPU time): the
    reference's CPU build on configurations 1-3 next to the GPU path on the same
    cases, 1 core pinned:
    * C1, the 24^3 hex cavity at Re 100: all 300 outer iterations;
    * C2, the k-epsilon CHT channel (256,000 + 51,200 cells) without the solid's
      volumetric source, which the reference cannot express: mean over outer
      iterations 2..20;
    * C3, the 2M-cell tet cavity: mean over outer iterations 2..10 of the -O3
      build, and outer iteration 1 of the reference's shipped -g build.
    Every solve at the configurations' 1e-8 with BiCGSTAB + Jacobi for momentum
    and scalars and Jacobi-CG for p' and the solid (both codes)."""
    from sysu_cfd_heat_gb300 import meshgen as mg
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    out = {"host": host_cpu()}

    def gpu_rate(param, iters, skip_first):
        with NavierStokesSolver(param, {"rtc": RTC}) as s:
            s.iterate(1)
            s.reset()
            if skip_first:
                s.iterate(1)
            s.timer_start()
            done = s.iterate(iters - (1 if skip_first else 0))
            ms = s.timer_stop()
        return done / (ms / 1000.0)

    with tempfile.TemporaryDirectory() as tmp:
        c1 = mg.write_case(os.path.join(tmp, "c1"), mg.lid_cavity_hex(24), mg.cavity_param("x", 300, mu=0.01))
        its, setup, err, rec = cpu_reference_run(c1, 300, 1e9, 3600)
        out["c1_cavity_24"] = {"cells": 13824, "cpu_iters_per_s": (len(its) / sum(its)) if its else None,
                               "cpu_sample": f"all {len(its) if its else 0} outer iterations", "cpu": rec,
                               "gpu_iters_per_s": gpu_rate(c1, 300, False), "error": err}
        c2 = mg.write_case(os.path.join(tmp, "c2"), mg.cht_channel(160, 40, 8, 40),
                           mg.cht_param("x", 20, nu=1e-5, k_solid=15.0))
        its, setup, err, rec = cpu_reference_run(c2, 20, 1e9, 3600)
        v, which = cpu_rate(its) if its else (None, "none")
        out["c2_cht_channel"] = {"cells": {"fluid": 256000, "solid": 51200}, "cpu_iters_per_s": v,
                                 "cpu_sample": which, "cpu": rec, "gpu_iters_per_s": gpu_rate(c2, 20, True),
                                 "gpu_sample": "mean over outer iterations 2..20", "error": err}
    c3 = case_dir("c3")
    its, setup, err, rec = cpu_reference_run(c3, 10, 1e9, 3600)
    v, which = cpu_rate(its) if its else (None, "none")
    itg, setup_g, errg, recg = cpu_reference_run(c3, 1, 1e9, 3600, build="g")
    out["c3_tet_cavity_2m"] = {"cells": 1996800, "cpu_iters_per_s": v, "cpu_sample": which, "cpu": rec,
                               "cpu_iteration_seconds": its, "reference_setup_s": setup,
                               "as_shipped_g_iters_per_s": (1.0 / itg[0]) if itg else None,
                               "as_shipped_g": recg, "error": err or errg}
    return out


def probe_p(args) -> dict:
    """--probe-p FORM (profiling runs, not part of the default run): on the C3 case,
    one outer iteration of the given p' form (after LEARN_ITERS training outer
    iterations for a learned form), then the momentum and p' solves of the next
    outer iteration once more; prints the time and iterations of both solves (the
    momentum in the form's precision).  The ncu summaries under profiles/ were
    captured from these runs."""
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    forms = {name: opts for name, opts, _ in P_FORMS}
    opts = dict(forms[args.probe_p])
    if args.host_loops:
        opts["graph_loops"] = 0  # per-kernel profiling: profilers skip kernels of graphs with conditional nodes
    with NavierStokesSolver(case_dir(args.workload), dict({"rtc": RTC, "timing": 1, "p.maxit": 100000}, **opts)) as s:
        if opts.get("p.learned"):
            s.set_option("p.learn_iters", LEARN_ITERS)
            s.set_option("p.learn_steps", LEARN_STEPS)
            s.iterate(LEARN_ITERS)
        s.iterate(1)
        s.CalculateVelocity()
        s.CalculatePressure()
        s.check()
        st = s.solve_stats()
        return {"form": args.probe_p, "p_ms": s.timing()[0], "p_iters": st["p"]["iters"][0],
                "p_status": st["p"]["status"][0], "mom_ms": s.timing()[1], "mom_iters": st["mom"]["iters"],
                "mom_status": st["mom"]["status"]}


def max_over_ranks(x: float, w: int) -> float:
    """The largest per-rank value over the ranks (gloo all-reduce): the timed region
    of a replica run ends when its slowest replica does."""
    if w <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_rate(w: int, steps: int, t_max_ms: float) -> float:
    """Whole-job outer iterations/s of w replicas that each ran `steps` iterations."""
    return w * steps / (t_max_ms / 1000.0)


def run_ours(args, r, w, lr):
    from sysu_cfd_heat_gb300 import _lib
    from sysu_cfd_heat_gb300.solver import NavierStokesSolver

    param = case_dir(args.workload) if r == 0 else None
    if w > 1:
        import torch.distributed as dist

        dist.barrier()
        param = case_dir(args.workload)
    L = _lib.lib()
    t_create = time.perf_counter()
    s = NavierStokesSolver(param, {"rtc": RTC, "timing": 1})
    t_create = time.perf_counter() - t_create
    ph = np.zeros(5)
    L.sysu_setup_phases(ph.ctypes.data_as(_lib.C.POINTER(_lib.C.c_double)))
    if args.p_maxit:
        s.set_option("p.maxit", args.p_maxit)
    if args.p_mixed:
        s.set_option("p.mixed", 1)
    info = s.info()
    n, nnz = info["Ncel"], info["nnz"]
    # warm-up, then back to the initial state so the timed iterations are iterations 1..K
    s.iterate(args.warmup)
    s.reset()
    if w > 1:
        dist.barrier()
    clk = ClockSampler(lr)
    clk.start()
    l0 = L.sysu_kernel_launches()
    s_ms = 0.0
    p_ms, cg_it, mom_it = [], [], []
    for k in range(args.steps):
        s.timer_start()
        done = s.iterate(1)
        ms = s.timer_stop()
        assert done == 1
        s_ms += ms
        pm, _ = s.timing()
        st = s.solve_stats()
        p_ms.append(pm)
        cg_it.append(st["p"]["iters"][0])
        mom_it.append(st["mom"]["iters"])
    launches = L.sysu_kernel_launches() - l0
    clocks = clk.stop()
    t_max = max_over_ranks(s_ms, w)
    if w > 1:
        dist.barrier()
    value = replicas_rate(w, args.steps, t_max)

    # end to end through the C ABI with host buffers (page-locked, so the copies are DMA)
    s.reset()
    state = ("U", "V", "W", "P", "RUFace")
    host = {}
    for f in state:
        host[f] = _lib.pinned_empty(s.field_size(f))
        s.get(f, out=host[f])
    h2d = sum(a.nbytes for a in host.values())
    d2h = h2d
    if w > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        for f, a in host.items():
            s.set(f, a)
        s.iterate(1)
        for f in state:
            s.get(f, out=host[f])
    e2e_s = max_over_ranks(time.perf_counter() - t0, w)

    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    # dominant kernel: the persistent p' CG launch (one per outer iteration)
    b_iter = cg_bytes_per_iter(n, nnz)
    init_b = nnz * 12 + 48 * n  # initial residual: matrix, x gathered, b, D^-1 read, r, z written
    bytes_launch = [it * b_iter + init_b for it in cg_it]
    ach = [b / (ms / 1000.0) / 1e9 for b, ms in zip(bytes_launch, p_ms) if ms > 0]
    achieved = statistics.mean(ach) if ach else None
    f_iter = cg_flops_per_iter(n, nnz)
    dp = [it * f_iter / (ms / 1000.0) / 1e12 for it, ms in zip(cg_it, p_ms) if ms > 0]
    dp_tflops = statistics.mean(dp) if dp else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "cg_pressure_traffic.json")
    if args.workload == "c3" and not args.p_mixed and os.path.exists(tp):
        tj = json.load(open(tp))
        per_iter = tj.get("dram_bytes_per_cg_iteration_scaled_to_c3")
        if per_iter:
            traffic = per_iter * statistics.mean(cg_it)

    forms = {"fp64": {"iters_per_s": value, "ms_per_step": t_max / args.steps,
                      "p_solve_ms_mean": statistics.mean(p_ms), "p_cg_iters_mean": statistics.mean(cg_it),
                      "p_maxit": 1000}}
    if not args.p_maxit and not args.p_mixed:
        forms["matched_1e-8"] = matched_forms(s, args, n, nnz, hbm)

    # the reference's own solver mode (GMRES(10) + SSOR, CG + SSOR), outer iteration 1
    if not args.p_maxit and not args.p_mixed:
        s.set_option("reference_solvers", 1)
        s.reset()
        s.timer_start()
        s.iterate(1)
        ms_ref = s.timer_stop()
        st = s.solve_stats()
        forms["reference_solver_mode_outer_iteration_1"] = {
            "ms": ms_ref, "solvers": "momentum GMRES(10)+SSOR(1.2) per component, p' CG+SSOR(1.3), level-scheduled",
            "mom_gmres_iters": st["mom"]["iters"], "p_cg_ssor_iters": st["p"]["iters"][0],
            "p_rel_residual": st["p"]["res"][0]}
        s.set_option("reference_solvers", 0)

    # standalone SpMV sweep on the assembled matrices after outer iterations 1, 10, 100
    forms["spmv_sweep"] = spmv_sweep(s, n, nnz, hbm) if not args.p_maxit and not args.p_mixed else None
    # the batched k, eps, T form needs a k-epsilon + energy case: not this cavity
    forms["batch_48_cavities"] = (batch_form(args) if args.workload == "c3" and not args.p_maxit
                                  and not args.p_mixed and not args.no_batch else None)
    forms["c2_cht_channel"] = (c2_form(args) if args.workload == "c3" and not args.p_maxit
                               and not args.p_mixed and not args.no_batch else None)

    out = {
        "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": w, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered-tet cavity)",
        "config": config_of(args),
        "e2e": {"value": w * args.steps / e2e_s, "unit": "iters/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_cg_pipe (persistent Jacobi-PCG for p')",
                     "achieved": achieved, "peak": hbm, "peak_source": peak_src, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                     "algorithmic_bytes_per_cg_iteration": b_iter},
        "fp64_pipe": {"kernel": "k_cg_pipe", "achieved_tflops": dp_tflops, "peak_tflops": FP64_PEAK_TFLOPS,
                      "peak_source": "nominal GB300 FP64 rate (2 FMA lanes per SM per clock)",
                      "frac": (dp_tflops / FP64_PEAK_TFLOPS) if dp_tflops else None,
                      "flops_per_cg_iteration": f_iter},
        "p_solve_ms_mean": statistics.mean(p_ms), "p_cg_iters_mean": statistics.mean(cg_it),
        "mom_bicgstab_iters": mom_it[-1], "clocks": clocks, "forms": forms,
        "setup": {"solver_create_s": t_create, "msh_read_s": ph[0], "faces_s": ph[1], "split_s": ph[2],
                  "geometry_s": ph[3], "host_threads": int(ph[4]),
                  "note": "solver creation = param.in + MSH read + faces + geometry + device upload; "
                          "topology and geometry are bit-identical for any thread count"},
    }
    s.close()
    if r == 0 and w == 1 and not args.no_cpu_baseline:
        its, setup, err, rec = cpu_reference_run(param, 3, args.cpu_budget, args.cpu_budget + 600)
        if setup is not None:
            out["setup"]["reference_setup_s"] = setup
        if its:
            nx, ny, nz = WORKLOADS[args.workload]
            v, which = cpu_rate(its)
            out["cpu_baseline"] = {"value": v, "unit": "iters/s", "cores": 1, "kind": "reference",
                                   "sample": f"{which} of the same {6 * nx * ny * nz}-cell case (reference C++ + "
                                             f"LASPack restatement, {rec['flags']}, 1 thread pinned to core "
                                             f"{rec['pinned_core']}, set-up {setup:.1f} s excluded)",
                                   "iteration_seconds": its, "host": rec}
        else:
            out["cpu_baseline"] = {"value": None, "unit": "iters/s", "cores": 1, "kind": "reference",
                                   "sample": err or "no iteration finished within the budget"}
    if r == 0:
        print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 48-cavity batch form")
    ap.add_argument("--learned-c5", action="store_true",
                    help="only the configuration-5 learned-preconditioner run (4.9 M cells; minutes)")
    ap.add_argument("--host-loops", action="store_true",
                    help="with --probe-p: the host drives the solves' loops (for per-kernel ncu captures)")
    ap.add_argument("--probe-p", default=None, choices=[f for f, _, _ in P_FORMS],
                    help="only one p' solve of the given form after its set-up (profiling runs)")
    ap.add_argument("--cpu-survey", action="store_true",
                    help="only the CPU baseline of configurations 1-3 next to the GPU (minutes of CPU time)")
    ap.add_argument("--cpu-budget", type=float, default=60.0,
                    help="seconds of reference outer iterations for the cpu_baseline sample (at most 3 iterations)")
    ap.add_argument("--ref-budget", type=float, default=900.0,
                    help="reference arm: stop early once its outer iterations add up to this many seconds")
    ap.add_argument("--p-maxit", type=int, default=0,
                    help="cap the p' CG iterations (short profiling runs only; not a bench setting)")
    ap.add_argument("--p-mixed", action="store_true",
                    help="time the mixed-precision p' form as the main form (profiling runs)")
    args = ap.parse_args()
    r, w, lr = rank_info()
    if w > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(lr))
        import torch.distributed as dist

        dist.init_process_group("gloo")
    if args.probe_p:
        if r == 0:
            print(json.dumps({"probe_p": probe_p(args)}))
    elif args.cpu_survey:
        if r == 0:
            print(json.dumps({"cpu_survey": cpu_survey(args)}))
    elif args.learned_c5:
        if r == 0:
            print(json.dumps({"learned_c5": c5_learned_run(args)}))
    elif args.impl == "reference":
        run_reference(args, r, w)
    else:
        run_ours(args, r, w, lr)
    if w > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

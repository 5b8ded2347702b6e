"""Benchmark of the DVM time step on GB300.

Workload: the 1-D normal shock -- 200 cells, 32^3 uniform velocity grid on [-9, 9],
variable-hard-sphere gas (omega = 0.81), Mach 3.0 Rankine-Hugoniot end states joined by a
tanh profile 10 upstream mean free paths wide, inflow Maxwellian conditions at both ends,
variance-reduced Monte Carlo collisions with 2e5 samples per cell-step, FP64. A step is
one solve() iteration: collisions in every cell, convection with the end conditions, and
the moments.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line. `value` is device-timed collisions/s with f resident in HBM (L2
flushed between timed steps); `e2e` runs the same steps through the C ABI with the
distribution in pinned host memory, copied in and out every step.
`--impl reference` times the CPU restatement of the reference's step (the Fortran
reference cannot be built here) on the host cores.
"""
import argparse
import ctypes as C
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

NCELLS = 200
NGRID = 32
VMAX = 9.0
MACH = 3.0
WIDTH = 10.0
DX = 0.5
DT = 0.05
OMEGA = 0.81
SAMPLES = 200000
SEED = 20261203
BYTES_PER_SAMPLE = 8 * (2 + 2 * 16)  # 2 partner reads + 16 atomic read-modify-writes
ATOMICS_PER_SAMPLE = 16              # 2 depletions + 2 x 7 replenishment nodes


def workload_config(pkg, ncells=None):
    global NCELLS
    if ncells:
        NCELLS = ncells
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(NGRID, -VMAX, VMAX)
    f0, up, dn = ph.shock_profile(g, NCELLS, DX, MACH, WIDTH)
    walls = ((dn["n"], dn["u"], 0.0, 0.0, dn["T"]), (up["n"], up["u"], 0.0, 0.0, up["T"]),
             (1.0, 0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 0.0, 1.0))
    mol = ph.molecule("Ar", ph.CSECTION_VHS)
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=NCELLS, dx=DX, deltat=DT, Kn=1.0,
                        mass=mol["mass"], omega=mol["omega"], alpha=mol["alpha"],
                        sigma=ph.cross_section(mol, ph.CSECTION_BIRD),
                        iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                        samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=SAMPLES,
                        bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 0, 0), walls=walls,
                        seed=SEED)
    return cfg, g, f0


def config_record(impl):
    return {
        "workload": "1-D normal shock: %d cells x %d^3 velocity grid on [-%g,%g], VHS omega=%g, "
                    "Mach %g, tanh profile %g mfp, inflow Maxwellian ends, VR collisions "
                    "%d samples/cell-step, FP64" % (NCELLS, NGRID, VMAX, VMAX, OMEGA, MACH,
                                                    WIDTH, SAMPLES),
        "cells": NCELLS, "velocity_nodes": NGRID ** 3, "samples_per_cell_step": SAMPLES,
        "dt": DT, "dx": DX, "l2": "flushed (256 MiB write) between timed steps" if impl == "gpu"
        else "n/a (CPU)",
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def dist_reduce(dist, value, op):
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


# -----------------------------------------------------------------------------------------
def cpu_rate(oracle, pkg, cfg, g, f0, threads, budget_s, cells_cap=NCELLS):
    """Collisions/s of the CPU restatement on a bounded sample of the workload: the first
    n cells of the shock (n sized to the time budget), full steps (collisions, convection,
    moments) run with `threads` OpenMP threads."""
    import dataclasses
    cells_cap = min(cells_cap, len(f0))
    probe_cells = min(8, cells_cap)
    sub = dataclasses.replace(cfg, nx_space=probe_cells)
    s = oracle.OracleSolver(sub, g, threads=threads)
    s.initialize_dist_func(f0[:probe_cells])
    t0 = time.perf_counter()
    s.solve(1)
    t_probe = time.perf_counter() - t0
    per_cell = t_probe / probe_cells
    n = int(max(probe_cells, min(cells_cap, budget_s / max(per_cell, 1e-9))))
    if n > probe_cells:
        sub = dataclasses.replace(cfg, nx_space=n)
        s = oracle.OracleSolver(sub, g, threads=threads)
        s.initialize_dist_func(f0[:n])
    t0 = time.perf_counter()
    s.solve(1)
    dt = time.perf_counter() - t0
    colls = s.collision_count()
    return colls / dt, n, dt


def run_reference(args):
    ws, rank, _ = dist_env()
    dist = dist_init(ws)
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    O.build()
    pkg = importlib.import_module("2d_dvm_microflows_gb300")
    cfg, g, f0 = workload_config(pkg, args.cells)
    threads = O.lib().orc_max_threads()
    # one untimed step to size the per-step sample (cells) to ~20 s per step at most
    rate, ncells, _ = cpu_rate(O, pkg, cfg, g, f0, threads, budget_s=20.0)
    import dataclasses
    sub = dataclasses.replace(cfg, nx_space=ncells)
    s = O.OracleSolver(sub, g, threads=threads)
    s.initialize_dist_func(f0[:ncells])
    for _ in range(args.warmup):
        s.solve(1)
    colls, t_total = 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s.solve(1)
        t_total += time.perf_counter() - t0
        colls += s.collision_count()
    value = colls / t_total
    sample = ("first %d of %d cells of the workload per step (full steps: collisions, "
              "convection, moments), %d timed steps" % (ncells, NCELLS, args.steps))
    line = {
        "impl": "reference", "metric": "MC collisions/s", "value": value, "unit": "collisions/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded R-H tanh shock state)",
        "config": config_record("cpu"),
        "cpu_baseline": {"value": value, "unit": "collisions/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "collisions/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference step (oracle/), OpenMP over cells; the "
                "Fortran reference has no compiler in this image",
    }
    print(json.dumps(line))
    return 0


def time_steps(s, steps, warmup, kernels=None):
    """Device time of `steps` steps (L2 flushed before each, warm-up first): returns
    (collisions per second, ms per step); per-kernel event times go into `kernels`."""
    for _ in range(warmup):
        s.solve(1)
    s.synchronize()
    s.profile_reset()
    t, colls = 0.0, 0
    for _ in range(steps):
        s.profile(False)
        s.flush_l2()
        s.synchronize()
        s.profile(True)
        t += s.time_steps(1)
        colls += s.collision_count()
    s.profile(False)
    if kernels is not None:
        kernels.update({k: round(v[0] / max(v[1], 1), 4)
                        for k, v in s.profile_read().items() if v[1]})
    return colls / (t * 1e-3), t / steps


def moment_error(p_test, p_ref):
    """Per moment field, max over cells of |test - ref| / the field's physical scale
    (n; sqrt(T) for velocities; T; p for stresses; n T^1.5 for heat flux)."""
    n, T = np.abs(p_ref[:, 0]).max(), np.abs(p_ref[:, 4]).max()
    pr = 0.5 * n * T
    sc = np.array([n, T ** 0.5, T ** 0.5, T ** 0.5, T, T, T ** 0.5, pr] + [n * T ** 1.5] * 3 +
                  [pr] * 6)
    e = np.abs(p_test[:, :17] - p_ref[:, :17]).max(0) / sc
    return {"max": float(e.max()),
            "per_field": {k: float(v) for k, v in zip(
                ["dens", "u", "v", "w", "temp", "species_temp", "avg_speed", "pressure", "qx",
                 "qy", "qz", "txx", "tyy", "tzz", "txy", "txz", "tyz"], e)}}


ENS_SEEDS = 4  # independent seeds per precision in the ensemble accuracy comparisons


def ensemble_error(pkg, make, steps, seeds=ENS_SEEDS):
    """Accuracy of the precision form against FP64 at matched ensembles:
    `make(precision, seed)` returns a stepped-ready solver (or batch); after `steps` steps the
    means over `seeds` independent seeds of each precision are compared per moment field
    (moment_error), beside the FP64 ensemble's own standard error on the same scale."""
    ens = {}
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        runs = []
        for k in range(seeds):
            s = make(prec, SEED + 7919 * (k + 1))
            s.step(steps) if hasattr(s, "upload_f") else s.solve(steps)
            runs.append(s.properties())
            s.close()
        ens[prec] = np.array(runs)
    m64 = ens[pkg.DVM_PREC_FP64].mean(0)
    se = ens[pkg.DVM_PREC_FP64].std(0, ddof=1) / np.sqrt(seeds)
    out = moment_error(ens[pkg.DVM_PREC_FP32].mean(0), m64)
    out["fp64_ensemble_standard_error_max"] = moment_error(m64 + se, m64)["max"]
    out["seeds"] = seeds
    out["steps"] = steps
    return out


def cavity_config(pkg):
    """2-D microcavity: 64 x 64 cells (unit side), 24^3 grid on [-5, 5], hard sphere,
    Kn = 0.1, three diffuse walls at T = 1, lid diffuse at T = 1 moving at u = 0.3,
    rest Maxwellian start, samples per cell-step from the reference formula (ColnRMS 0.001)."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(24, -5.0, 5.0)
    mol = ph.molecule("Ar", ph.CSECTION_HS)
    n = 64
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_2D, nx_space=n, ny_space=n, dx=1.0 / n,
                        dy=1.0 / n, deltat=0.0025, Kn=0.1, mass=1.0, omega=mol["omega"],
                        alpha=mol["alpha"], sigma=ph.cross_section(mol, ph.CSECTION_BIRD),
                        iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1, ColnRMS=0.001,
                        samples_mode=pkg.DVM_SAMPLES_FORMULA, acc_coeff=1.0, walls=walls,
                        seed=SEED)
    f0 = np.tile(ph.maxwellian(g, 1.0, 0.0, 0.0, 0.0, 1.0), (n * n, 1))
    return cfg, g, f0


def run_forms(pkg, args, fp64_value):
    """The precision form (FP32 sampling/scatter + FP64 projection) on the shock workload
    and on the 2-D cavity, each beside the FP64 plain method from the same start and seed."""
    import dataclasses
    out = {}
    cfg, g, f0 = workload_config(pkg, args.cells)

    def make(prec, seed):
        s = pkg.DVMSolver(dataclasses.replace(cfg, precision=prec, seed=seed), g)
        s.initialize_dist_func(f0)
        return s
    res = {}
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        s = pkg.DVMSolver(dataclasses.replace(cfg, precision=prec), g)
        s.initialize_dist_func(f0)
        rate, ms = time_steps(s, args.steps, args.warmup)
        res[prec] = (rate, ms, s.properties())
        s.close()
    out["fp32_shock"] = {
        "value": res[pkg.DVM_PREC_FP32][0], "unit": "collisions/s",
        "ms_per_step": res[pkg.DVM_PREC_FP32][1],
        "fp64_value_same_run": res[pkg.DVM_PREC_FP64][0],
        "speedup_vs_fp64": res[pkg.DVM_PREC_FP32][0] / res[pkg.DVM_PREC_FP64][0],
        "moment_err_ensemble_vs_fp64": ensemble_error(pkg, make, 8)}
    out["cavity"] = run_cavity(pkg, args)
    return out


def one_step_error(pkg, cfg, g, f0, steps_before=3):
    """The precision form's own error: from one FP64 state, one FP64 step and one FP32 step
    with the same Philox words (hence the same partners), compared per moment field."""
    import dataclasses
    s = pkg.DVMSolver(dataclasses.replace(cfg, precision=pkg.DVM_PREC_FP64), g)
    s.initialize_dist_func(f0)
    s.solve(steps_before)
    state = s.phi()
    s.close()
    out = []
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        s = pkg.DVMSolver(dataclasses.replace(cfg, precision=prec), g)
        s.initialize_dist_func(state)
        s.ntime = steps_before
        s.solve(1)
        out.append(s.properties())
        s.close()
    return moment_error(out[1], out[0])


def run_cavity(pkg, args):
    """The 2-D microcavity in the precision form and in FP64 from the same start and seed."""
    import dataclasses
    cfg, g, f0 = cavity_config(pkg)
    res = {}
    kern = {}
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        s = pkg.DVMSolver(dataclasses.replace(cfg, precision=prec), g)
        s.initialize_dist_func(f0)
        kern[prec] = {}
        rate, ms = time_steps(s, args.steps, args.warmup, kern[prec])
        res[prec] = (rate, ms, s.properties(), s.collision_count())
        s.close()
    cells = cfg.nx_space * cfg.ny_space
    one_step = one_step_error(pkg, cfg, g, f0)

    def make(prec, seed):
        s = pkg.DVMSolver(dataclasses.replace(cfg, precision=prec, seed=seed), g)
        s.initialize_dist_func(f0)
        return s
    return {
        "one_step_moment_err_fp32_vs_fp64": one_step,
        "workload": "2-D microcavity 64x64 cells, 24^3 on [-5,5], hard sphere, Kn=0.1, "
                    "diffuse walls T=1, lid u=0.3, samples from the reference formula "
                    "(ColnRMS 0.001), dt=0.0025",
        "collisions_per_step": res[pkg.DVM_PREC_FP32][3],
        "fp32": {"value": res[pkg.DVM_PREC_FP32][0], "unit": "collisions/s",
                 "ms_per_step": res[pkg.DVM_PREC_FP32][1],
                 "cell_updates_per_s": cells / (res[pkg.DVM_PREC_FP32][1] * 1e-3),
                 "ms_per_launch": kern[pkg.DVM_PREC_FP32]},
        "fp64": {"value": res[pkg.DVM_PREC_FP64][0], "unit": "collisions/s",
                 "ms_per_step": res[pkg.DVM_PREC_FP64][1],
                 "cell_updates_per_s": cells / (res[pkg.DVM_PREC_FP64][1] * 1e-3),
                 "ms_per_launch": kern[pkg.DVM_PREC_FP64]},
        "moment_err_ensemble_vs_fp64": ensemble_error(pkg, make, 8)}


BATCH_GRIDS = (16, 24, 32, 40)
BATCH_INSTANCES = 256
BATCH_SAMPLES_24 = 100000  # samples per instance-step on 24^3; proportional to N_v


def batch_workload(pkg, ninst=BATCH_INSTANCES, seed=SEED):
    """256 homogeneous relaxations: grids drawn uniformly from {16,24,32,40}^3 on [-5,5],
    bimodal starts (weights 1/2, temperature ratio ~U[1,4], x-drift +-U[0,1.5]), samples per
    step 1e5 * N_v / 24^3."""
    ph = pkg.physics
    grids = [ph.VelocityGrid.uniform(n, -5.0, 5.0) for n in BATCH_GRIDS]
    samples = [int(BATCH_SAMPLES_24 * (n / 24.0) ** 3) for n in BATCH_GRIDS]
    rng = np.random.default_rng(seed)
    gid = rng.integers(0, len(grids), ninst).astype(np.int32)
    f0 = []
    for i in range(ninst):
        g = grids[gid[i]]
        tr, u = rng.uniform(1.0, 4.0), rng.uniform(0.0, 1.5)
        f0.append(0.5 * ph.maxwellian(g, 1.0, u, 0.0, 0.0, 1.0) +
                  0.5 * ph.maxwellian(g, 1.0, -u, 0.0, 0.0, tr))
    cfg = pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, deltat=0.01, seed=seed)
    return cfg, grids, gid, samples, f0


def run_batch(pkg, args):
    """The batched form (one CUDA-graph replay per step over all instances, autotuned
    persistent launches) in FP32+projection and FP64, beside the plain FP64 path that steps
    each instance through its own context, one dvm_step call per instance-step."""
    import dataclasses
    cfg, grids, gid, samples, f0 = batch_workload(pkg)
    per_step = int(sum(samples[q] for q in gid))
    out = {"workload": "%d homogeneous relaxations, grids {16,24,32,40}^3 on [-5,5], bimodal "
                       "T-ratio U[1,4], drift U[0,1.5], VR hard sphere, dt 0.01, samples "
                       "1e5*N_v/24^3 per instance-step" % len(gid),
           "collisions_per_step": per_step,
           "grid_counts": {"%d^3" % n: int((gid == q).sum()) for q, n in enumerate(BATCH_GRIDS)}}
    props = {}
    for name, prec in (("fp32_batched", pkg.DVM_PREC_FP32), ("fp64_batched", pkg.DVM_PREC_FP64)):
        b = pkg.DVMBatch(dataclasses.replace(cfg, precision=prec), grids, gid, samples)
        for i, f in enumerate(f0):
            b.upload_f(i, f)
        b.step(args.warmup)  # capture, autotune and warm up
        ms_dev, colls = b.time_steps(args.steps)
        t0 = time.perf_counter()
        b.step(args.steps)
        b.properties()
        wall = time.perf_counter() - t0
        props[name] = b.properties()
        out[name] = {"value": colls / (ms_dev * 1e-3), "unit": "collisions/s",
                     "ms_per_step": ms_dev / args.steps,
                     "wall_collisions_per_s": per_step * args.steps / wall,
                     "instance_updates_per_s": len(gid) * args.steps / wall,
                     "launch_shape": b.launch_shape()}
        b.close()

    def make(prec, seed):
        b = pkg.DVMBatch(dataclasses.replace(cfg, precision=prec, seed=seed), grids, gid, samples)
        for i, f in enumerate(f0):
            b.upload_f(i, f)
        return b
    out["moment_err_ensemble_fp32_vs_fp64"] = ensemble_error(pkg, make, 2 * args.steps +
                                                             args.warmup, seeds=3)
    one = []
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        b = pkg.DVMBatch(dataclasses.replace(cfg, precision=prec), grids, gid, samples)
        for i, f in enumerate(f0):
            b.upload_f(i, f)
        b.step(1)
        one.append(b.properties())
        b.close()
    out["one_step_moment_err_fp32_vs_fp64"] = moment_error(one[1], one[0])
    out["note"] = ("moment_err_ensemble_* compares ensemble means over independent seeds; "
                   "one_step_* isolates the FP32 rounding: one step of each form from the "
                   "same state and Philox words")
    # plain FP64: one context per instance, stepped one after another
    solvers = []
    for i, f in enumerate(f0):
        c = dataclasses.replace(cfg, samples_mode=pkg.DVM_SAMPLES_FIXED,
                                samples_per_step=samples[gid[i]])
        s = pkg.DVMSolver(c, grids[gid[i]])
        s.initialize_dist_func(f)
        solvers.append(s)
    for s in solvers:
        s.solve(1)
    for s in solvers:
        s.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in solvers:
            s.solve(1)
    for s in solvers:
        s.synchronize()
    wall = time.perf_counter() - t0
    out["fp64_plain"] = {"value": per_step * args.steps / wall, "unit": "collisions/s",
                         "ms_per_step": wall * 1e3 / args.steps,
                         "instance_updates_per_s": len(gid) * args.steps / wall}
    for s in solvers:
        s.close()
    out["speedup_fp32_batched_vs_fp64_plain"] = (out["fp32_batched"]["wall_collisions_per_s"] /
                                                 out["fp64_plain"]["value"])
    out["timing"] = ("batched value: CUDA events around graph replays (one grouped launch of "
                     "each kernel per step, launch_shape); wall_*: host clock around the same "
                     "replays; fp64_plain: host clock; working set > L2")
    return out


BATCH1D_INSTANCES = 64
BATCH1D_CELLS = 100
BATCH1D_SAMPLES = 20000  # per cell-step


def run_batch_1d(pkg, args):
    """1-D instances batched: 64 shock solves of 100 cells on 24^3 and 28^3 grids (Mach
    U[1.5,3] tanh profiles, one shared pair of inflow ends, 2e4 VR samples per cell-step),
    FP32+projection batched against the plain FP64 path (one context per instance, one
    dvm_step call per instance-step)."""
    import dataclasses
    ph = pkg.physics
    rng = np.random.default_rng(SEED + 1)
    grids = [ph.VelocityGrid.uniform(n, -8.0, 8.0) for n in (24, 28)]
    gid = rng.integers(0, len(grids), BATCH1D_INSTANCES).astype(np.int32)
    mol = ph.molecule("Ar", ph.CSECTION_VHS)
    f0 = []
    for i in range(BATCH1D_INSTANCES):
        f, up, dn = ph.shock_profile(grids[gid[i]], BATCH1D_CELLS, 0.5, rng.uniform(1.5, 3.0), 10.0)
        f0.append(f)
    _, up, dn = ph.shock_profile(grids[0], 3, 0.5, 2.0, 10.0)
    walls = ((dn["n"], dn["u"], 0.0, 0.0, dn["T"]), (up["n"], up["u"], 0.0, 0.0, up["T"]),
             (1.0, 0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 0.0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=BATCH1D_CELLS, dx=0.5, deltat=0.04,
                        Kn=1.0, mass=mol["mass"], omega=mol["omega"], alpha=mol["alpha"],
                        sigma=ph.cross_section(mol, ph.CSECTION_BIRD), iColl=pkg.DVM_COLL_VR,
                        iConv=pkg.DVM_CONV_UPWIND1, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=BATCH1D_SAMPLES,
                        bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 0, 0), walls=walls, seed=SEED)
    per_step = BATCH1D_INSTANCES * BATCH1D_CELLS * BATCH1D_SAMPLES
    out = {"workload": "%d 1-D shocks of %d cells on 24^3/28^3 grids on [-8,8], VHS, Mach "
                       "U[1.5,3], inflow ends, %d VR samples per cell-step"
                       % (BATCH1D_INSTANCES, BATCH1D_CELLS, BATCH1D_SAMPLES),
           "collisions_per_step": per_step}
    b = pkg.DVMBatch(dataclasses.replace(cfg, precision=pkg.DVM_PREC_FP32), grids, gid,
                     [BATCH1D_SAMPLES] * len(grids))
    for i, f in enumerate(f0):
        b.upload_f(i, f)
    b.step(args.warmup + 1)
    ms_dev, colls = b.time_steps(2 * args.steps)
    t0 = time.perf_counter()
    b.step(2 * args.steps)
    b.properties()
    wall = time.perf_counter() - t0
    out["fp32_batched"] = {"value": colls / (ms_dev * 1e-3), "unit": "collisions/s",
                           "ms_per_step": ms_dev / (2 * args.steps),
                           "wall_collisions_per_s": per_step * 2 * args.steps / wall,
                           "cell_updates_per_s": BATCH1D_INSTANCES * BATCH1D_CELLS * 2 *
                           args.steps / wall, "launch_shape": b.launch_shape()}
    b.close()
    solvers = []
    for i, f in enumerate(f0):
        s = pkg.DVMSolver(cfg, grids[gid[i]])
        s.initialize_dist_func(f)
        solvers.append(s)
    for s in solvers:
        s.solve(1)
    for s in solvers:
        s.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in solvers:
            s.solve(1)
    for s in solvers:
        s.synchronize()
    wall = time.perf_counter() - t0
    out["fp64_plain"] = {"value": per_step * args.steps / wall, "unit": "collisions/s",
                         "cell_updates_per_s": BATCH1D_INSTANCES * BATCH1D_CELLS * args.steps /
                         wall}
    bad = sum(int(s.error_word() != 0) for s in solvers)
    for s in solvers:
        s.close()
    out["fp64_plain"]["instances_with_error"] = bad
    out["speedup_fp32_batched_vs_fp64_plain"] = (out["fp32_batched"]["wall_collisions_per_s"] /
                                                 out["fp64_plain"]["value"])
    return out


SERVE_REQUESTS = 200
SERVE_RATE = 50.0        # Poisson arrivals per second
SERVE_MAX_STEPS = 40
SERVE_TOL = 1e-6
SERVE_BUDGET = 64 << 30  # admission budget, bytes of HBM
SERVE_SLOTS = 6   # concurrent requests (measured: 4.98e9 collisions/s at 6, 4.85e9 at 4 and 8)
SERVE_QUANTUM = 16   # steps per turn at most (the turn's graph loops on the device and
                     # stops at convergence; measured on 120 requests: 7.58e9 collisions/s
                     # at 16, 7.43e9 at 8, 6.80e9 at 40)
SERVE_PREEMPT = 0    # turns before a request yields its slot to a waiting one (0: never)
SERVE_ENS = 8        # seeds per precision in the ensemble accuracy comparison
SERVE_ENS_REQ = 3    # requests of each kind in that comparison


def serving_workload(pkg, nreq=SERVE_REQUESTS, seed=SEED):
    """Poisson arrivals (50 req/s) of mixed requests: 60% 1-D shocks (Mach ~U[1.2,4],
    100-400 cells, 24^3-32^3 grids, 2e4 samples per cell-step), 40% 2-D lid-driven cavities
    (Kn ~logU[0.01,1], 32x32-96x96 cells, 16^3-24^3 grids, 4e3 x max(1, 0.1/Kn) samples per
    cell-step: the weight of one sample grows as dt/Kn, and at Kn = 0.015 with 4e3 samples the
    Monte Carlo noise drives f negative and the state non-finite within 90 steps, so the count
    grows with 1/Kn as the reference's own formula makes it, compute_num_coll_pairs).
    Returns [(arrival_s, config, grid, f0, kind)] in arrival order."""
    ph = pkg.physics
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    mol = ph.molecule("Ar", ph.CSECTION_VHS)
    for i in range(nreq):
        t += rng.exponential(1.0 / SERVE_RATE)
        if rng.random() < 0.6:
            mach = rng.uniform(1.2, 4.0)
            cells = int(rng.integers(100, 401))
            n = int(rng.choice([24, 28, 32]))
            vmax = 4.0 + 1.6 * mach
            g = ph.VelocityGrid.uniform(n, -vmax, vmax)
            f0, up, dn = ph.shock_profile(g, cells, 0.5, mach, 10.0)
            walls = ((dn["n"], dn["u"], 0.0, 0.0, dn["T"]), (up["n"], up["u"], 0.0, 0.0, up["T"]),
                     (1.0, 0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 0.0, 1.0))
            cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=cells, dx=0.5,
                                deltat=0.9 * 0.5 / vmax, Kn=1.0, mass=mol["mass"],
                                omega=mol["omega"], alpha=mol["alpha"],
                                sigma=ph.cross_section(mol, ph.CSECTION_BIRD),
                                iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                                samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=20000,
                                bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 0, 0), walls=walls,
                                seed=seed + i)
            kind = "shock M=%.2f %d cells %d^3" % (mach, cells, n)
        else:
            kn = 10.0 ** rng.uniform(-2.0, 0.0)
            side = int(rng.choice([32, 48, 64, 80, 96]))
            n = int(rng.choice([16, 20, 24]))
            g = ph.VelocityGrid.uniform(n, -5.0, 5.0)
            f0 = np.tile(ph.maxwellian(g, 1.0, 0.0, 0.0, 0.0, 1.0), (side * side, 1))
            walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
            cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_2D, nx_space=side, ny_space=side,
                                dx=1.0 / side, dy=1.0 / side, deltat=0.9 / (side * 5.0 * 2.0),
                                Kn=kn, iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                                samples_mode=pkg.DVM_SAMPLES_FIXED,
                                samples_per_step=int(round(4000 * max(1.0, 0.1 / kn))),
                                walls=walls, seed=seed + i)
            kind = "cavity Kn=%.3f %dx%d %d^3" % (kn, side, side, n)
        out.append((t, cfg, g, f0, kind))
    return out


def _pct(v, q):
    return float(np.percentile(np.asarray(v), q))


def run_serving(pkg, args):
    """The served stream through the native request server (FP32+projection, continuous
    batching, admission by footprint) beside the plain FP64 path (one solve at a time in
    arrival order, a FIFO queue: latency = wait + service, service timed for real)."""
    import dataclasses
    reqs = serving_workload(pkg)
    # served: submissions at their arrival times
    served = []
    with pkg.DVMServer(SERVE_BUDGET, max_active=SERVE_SLOTS, steps_per_turn=SERVE_QUANTUM,
                       preempt_turns=SERVE_PREEMPT) as sv:
        t0 = time.perf_counter()
        ids = []
        for t, cfg, g, f0, _ in reqs:
            dt = t0 + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids.append(sv.submit(dataclasses.replace(cfg, precision=pkg.DVM_PREC_FP32), g, f0,
                                 SERVE_MAX_STEPS, SERVE_TOL))
        failed = []
        for rid, req in zip(ids, reqs):
            info = sv.wait(rid)
            try:
                props, _ = sv.result(rid)
            except pkg.DVMError as e:  # reported in the line, kept out of the statistics
                failed.append({"request": req[4], "error": str(e)})
                continue
            served.append((info, props, req))
        t_end = time.perf_counter()
        stats = sv.stats()
    window = t_end - t0
    colls = sum(i["collisions"] for i, _, _ in served)
    cells = sum((r[1].nx_space * r[1].ny_space) * i["steps"] for i, _, r in served)
    lat = [i["latency_ms"] for i, _, _ in served]
    out = {"workload": "%d requests, Poisson %.0f req/s: 60%% 1-D shocks (Mach U[1.2,4], "
                       "100-400 cells, 24^3-32^3, 2e4 samples/cell-step), 40%% 2-D cavities "
                       "(Kn logU[0.01,1], 32^2-96^2 cells, 16^3-24^3, 4e3 x max(1, 0.1/Kn) "
                       "samples/cell-step); "
                       "each to residual %g or %d steps" % (len(reqs), SERVE_RATE, SERVE_TOL,
                                                            SERVE_MAX_STEPS),
           "served_fp32": {"p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
                           "collisions_per_s": colls / window,
                           "cell_updates_per_s": cells / window,
                           "requests_per_s": len(reqs) / window,
                           "converged": sum(i["converged"] for i, _, _ in served),
                           "failed": failed,
                           "peak_active": stats["peak_active"],
                           "peak_bytes": stats["peak_bytes"], "budget_bytes": SERVE_BUDGET,
                           "statuses": sorted(set(i["status"] for i, _, _ in served))}}
    out["served_fp32"]["final_residual"] = {
        "median": _pct([i["residual"] for i, _, _ in served], 50),
        "max": max(i["residual"] for i, _, _ in served)}
    # plain FP64 under the same arrival clock: one solve at a time in arrival order, each
    # started when it has arrived and the previous one has finished; latency = finish -
    # arrival on the wall clock
    lat_p, colls_p, cells_p, resid_p, failed_p = [], 0, 0, [], 0
    t0 = time.perf_counter()
    for t, cfg, g, f0, _ in reqs:
        wait = t0 + t - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        s = pkg.DVMSolver(cfg, g)
        s.initialize_dist_func(f0)
        steps = 0
        while steps < SERVE_MAX_STEPS:
            s.solve(1)
            steps += 1
            colls_p += s.collision_count()
            if s.residual() <= SERVE_TOL:
                break
        resid_p.append(s.residual())
        failed_p += int(s.error_word() != 0)
        s.close()
        lat_p.append((time.perf_counter() - (t0 + t)) * 1e3)
        cells_p += cfg.nx_space * cfg.ny_space * steps
    span = time.perf_counter() - t0
    out["plain_fp64"] = {"p50_ms": _pct(lat_p, 50), "p99_ms": _pct(lat_p, 99),
                         "collisions_per_s": colls_p / span, "cell_updates_per_s": cells_p / span,
                         "requests_per_s": len(reqs) / span,
                         "converged": sum(1 for r in resid_p if r <= SERVE_TOL),
                         "failed": failed_p,
                         "final_residual": {"median": _pct(resid_p, 50), "max": max(resid_p)}}
    # accuracy at matched ensembles: the precision form the server runs (a request's result
    # depends only on its parameters, seed and steps) against FP64, SERVE_ENS seeds each, on
    # the first requests of each kind; errors are of the ensemble means, with the FP64
    # ensemble's own standard error beside them
    subset = ([r for r in reqs if r[4].startswith("shock")][:SERVE_ENS_REQ] +
              [r for r in reqs if r[4].startswith("cavity")][:SERVE_ENS_REQ])
    errs, ses = [], []
    for t, cfg, g, f0, _ in subset:
        ens = {}
        for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
            runs = []
            for k in range(SERVE_ENS):
                s = pkg.DVMSolver(dataclasses.replace(cfg, precision=prec,
                                                      seed=cfg.seed + 7919 * (k + 1)), g)
                s.initialize_dist_func(f0)
                s.solve(SERVE_MAX_STEPS)
                runs.append(s.properties())
                s.close()
            ens[prec] = np.array(runs)
        m64 = ens[pkg.DVM_PREC_FP64].mean(0)
        errs.append(moment_error(ens[pkg.DVM_PREC_FP32].mean(0), m64))
        se = ens[pkg.DVM_PREC_FP64].std(0, ddof=1) / np.sqrt(SERVE_ENS)
        ses.append(moment_error(m64 + se, m64))
    fields = errs[0]["per_field"].keys()
    out["moment_err_ensemble_fp32_vs_fp64"] = {
        "max": max(e["max"] for e in errs),
        "per_field": {k: max(e["per_field"][k] for e in errs) for k in fields},
        "fp64_ensemble_standard_error_max": max(e["max"] for e in ses),
        "requests": len(subset), "seeds": SERVE_ENS, "steps": SERVE_MAX_STEPS}
    out["note"] = ("each request runs to the residual or the step cap; the per-step residual "
                   "of a Monte Carlo step settles at the noise of the collision integral "
                   "(final_residual), far above 1e-6 at these sample counts. Accuracy is "
                   "compared between ensemble means of the precision form and of FP64 over "
                   "independent seeds, with the FP64 ensemble's standard error beside it")
    out["speedup_collisions"] = (out["served_fp32"]["collisions_per_s"] /
                                 out["plain_fp64"]["collisions_per_s"])
    out["speedup_cell_updates"] = (out["served_fp32"]["cell_updates_per_s"] /
                                   out["plain_fp64"]["cell_updates_per_s"])
    return out


def run_gpu(args):
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = dist_init(ws)
    import torch
    pkg = importlib.import_module("2d_dvm_microflows_gb300")
    cfg, g, f0 = workload_config(pkg, args.cells)
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    nv = g.nv
    # warm-up
    for _ in range(args.warmup):
        s.solve(1)
    s.synchronize()
    s.profile_reset()
    s.profile(True)
    launches0 = s.launch_count()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if ws > 1 else 0)
    dist_barrier(dist)
    clocks.start()
    t_dev, colls, scat = 0.0, 0, 0
    for _ in range(args.steps):
        s.profile(False)
        s.flush_l2()
        s.synchronize()
        s.profile(True)
        t_dev += s.time_steps(1)
        colls += s.collision_count()
        scat += s.scatter_count()
    s.synchronize()
    clk = clocks.stop()
    prof = s.profile_read()
    launches = s.launch_count() - launches0
    s.profile(False)
    dist_barrier(dist)
    t_max = dist_reduce(dist, t_dev, "max")
    colls_all = dist_reduce(dist, colls, "sum")
    value = colls_all / (t_max * 1e-3)

    # end to end through the C ABI: f in pinned host memory, moved in and out every step
    host = torch.empty((NCELLS, nv), dtype=torch.float64, pin_memory=True)
    hnp = host.numpy()
    hnp[:] = s.phi()
    ptr = hnp.ctypes.data_as(C.POINTER(C.c_double))
    lib = s.lib
    dist_barrier(dist)
    t0 = time.perf_counter()
    e2e_colls = 0
    for k in range(args.steps):
        # f from pinned host memory in, one step, f back out to the same host buffer
        # (dvm_step_host: the device reads and writes the page-locked buffer in its moments
        # passes)
        if lib.dvm_step_host(s.ctx, C.c_uint64(10000 + k), 1, ptr, ptr):
            raise RuntimeError("step failed")
        e2e_colls += cfg.samples_per_step * NCELLS
    t_e2e = time.perf_counter() - t0
    t_e2e = dist_reduce(dist, t_e2e, "max")
    e2e_value = dist_reduce(dist, e2e_colls, "sum") / t_e2e
    err = s.error_word()

    if rank != 0:
        return 0
    # roofline of the dominant kernel (collide), from the live event timings
    ms_coll, n_coll = prof["collide"]
    samples_per_launch = SAMPLES * NCELLS
    t_launch = ms_coll / max(n_coll, 1) * 1e-3
    achieved = samples_per_launch * BYTES_PER_SAMPLE / t_launch / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tp = os.path.join(REPO, "profiles", "collide_traffic.json")
    if os.path.exists(tp):
        with open(tp) as fh:
            traffic = json.load(fh).get("bytes_per_launch")
    kernels = {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof.items() if v[1]}
    # the collide kernel's scatter is FP64 atomics into an L2-resident f: its second
    # roofline is the measured atomic rate over a window the size of f
    atom_peak = s.atomic_rate(NCELLS * nv * 8)
    # adds per launch as counted by the kernel itself (dvm_last_scatter_count)
    atom_per_sample = scat / max(colls, 1)
    atom_achieved = scat / max(args.steps, 1) / t_launch
    line = {
        "metric": "MC collisions/s", "value": value, "unit": "collisions/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded R-H tanh shock state)", "config": config_record("gpu"),
        "cell_updates_per_s": NCELLS * args.steps * ws / (t_max * 1e-3),
        # the collide kernel's read-modify-writes stay in L2 (its DRAM traffic is about 1 %
        # of the bytes it moves), so the roofline that bounds it is the L2 FP64 atomic rate;
        # the HBM view is kept beside it with the measured traffic
        "roofline": {"bound": "l2_atomic", "kernel": "collide", "achieved": atom_achieved,
                     "peak": atom_peak, "unit": "FP64 atomic adds/s",
                     "frac": atom_achieved / atom_peak, "traffic": traffic,
                     "atomics_per_sample": atom_per_sample,
                     "atomics_per_sample_source": "counted by the collide kernel",
                     "atomics_per_sample_nominal": ATOMICS_PER_SAMPLE,
                     "peak_source": "measured in this run (dvm_atomic_rate, pseudo-random "
                                    "FP64 adds over a window the size of f)"},
        "roofline_hbm": {"bound": "hbm", "kernel": "collide", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind, "traffic": traffic,
                         "traffic_over_algorithmic": (traffic / (samples_per_launch *
                                                                 BYTES_PER_SAMPLE)
                                                      if traffic else None),
                         "algorithmic_bytes_per_sample": BYTES_PER_SAMPLE},
        "kernels": kernels,
        "e2e": {"value": e2e_value, "unit": "collisions/s",
                "h2d_bytes_per_step": NCELLS * nv * 8, "d2h_bytes_per_step": NCELLS * nv * 8},
        "gpu_launches": launches,
        "clocks": clk,
        "error_word": err,
    }
    if ws == 1 and not args.no_forms:
        line["forms"] = run_forms(pkg, args, value)
        line["forms"]["batched"] = run_batch(pkg, args)
        line["forms"]["batched_1d"] = run_batch_1d(pkg, args)
        line["forms"]["served"] = run_serving(pkg, args)
    if ws == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle as O
        O.build()
        rate, ncells, dt = cpu_rate(O, pkg, cfg, g, f0, 1, budget_s=12.0)
        line["cpu_baseline"] = {"value": rate, "unit": "collisions/s", "cores": 1, "kind": "port",
                                "sample": "one full step of the first %d of %d cells, single "
                                          "thread (%.1f s)" % (ncells, NCELLS, dt)}
    print(json.dumps(line))
    s.close()
    return 0


def run_case(args):
    """One form alone (for profiling and quick checks): prints its JSON object."""
    pkg = importlib.import_module("2d_dvm_microflows_gb300")
    fn = {"cavity": run_cavity, "batch": run_batch, "batch1d": run_batch_1d,
          "served": run_serving}[args.case]
    print(json.dumps({"case": args.case, "result": fn(pkg, args)}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the precision-form and cavity measurements")
    ap.add_argument("--cells", type=int, default=None,
                    help="smaller case of the same workload (profiling only)")
    ap.add_argument("--case", default=None, choices=["cavity", "batch", "batch1d", "served"],
                    help="run one form alone and print its result (profiling)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gpu":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.case:
        return run_case(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

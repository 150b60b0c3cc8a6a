#!/usr/bin/env python
"""Throughput of the Taylor-Couette time step on GB300, in Mcell-steps/s.

Workload (default, "C3"): 1024 x 768 x 512 (theta x z x r) cells, radial
clustering at both walls with the reference's own bou.in grid (ISTR=6,
STR3=20: the configuration's ISTR=1 is undefined in the reference grid
generator), RINT=1, REXT=1.4, ALX3D=2*pi, rotating frame ROTP=0.1,
1/NU=2e4, RK3, variable dt (CFLMAX=1.2, DTMIN=1e-5, DTMAX=1.8e-4), seeded
Couette-plus-noise start (amplitude 0.01).  One "step" is one full RK3 time
step (three substeps) with the dt rule of main.F90, FP64 throughout.
"C2" (512 x 512 x 384, oscillating inner cylinder, DTMAX 3e-4) is the
production-size case of the same path; "C1" the small CPU-runnable one.

  value  : steps with the state resident in HBM (tc_run, one host sync)
  e2e    : through the C ABI with host buffers: tc_set_state from page-locked
           host memory on huge pages (tc_host_alloc), one tc_run(1) per step
           (the host reads dt/time back each step, as the reference's host
           loop does), tc_get_state into the same kind of buffers at the end
  roofline: the kernel class with the largest share of the timed region,
           algorithmic HBM bytes per launch / its mean CUDA-event duration
  cpu_baseline: the CPU oracle (C++ restatement of the reference's serial
           algorithm) on the host cores, on a bounded sample of the workload
  mixed  : the same workload in the mixed FP32/FP64 form (FP64 pressure
           tridiagonals; the float-float variant beside it), with its error
           against the FP64 run after the same steps
  ensemble: the batched ensemble of 96 drawn instances, FP64 and mixed
  serving: continuous batching of Poisson arrivals at two rates, p50/p99

Under torchrun (N > 1) every rank advances its own replica (the time step of
one run does not shard without the reference's halo and transpose exchanges),
so scaling is weak and value sums the replicas.
``--impl reference`` times the CPU oracle alone on rank 0, on the full grid
of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DTMAX (not fixed by the configurations): the reference scheme also needs
# U dt / dr_min below about 2-4 (the explicit product-rule part of the radial
# flux d(qr qt)/dr, which CalcMaxCFL does not measure); on the clustered grids
# below dt = 1e-3 grows a mode from roundoff within 20 steps (CPU oracle and
# GPU alike), so DTMAX keeps U dt / dr_min near 1.3.
WORKLOADS = {
    "C2": dict(nthm=512, nzm=512, nrm=384, istr=6, str=20.0, ren=5000.0, sizepert=0.1, omegapert=0.5,
               idtv=1, limitCFL=1.2, dtmin=1e-5, dtmax=3e-4),
    "C1": dict(nthm=64, nzm=64, nrm=64, istr=0, ren=1000.0, idtv=1, limitCFL=1e3, dtmin=1e-3, dtmax=1e-3),
    # profiling size: the C2 theta-z plane with a third of the radial cells (a few GB on the device)
    "P2": dict(nthm=512, nzm=512, nrm=128, istr=6, str=20.0, ren=5000.0, sizepert=0.1, omegapert=0.5,
               idtv=1, limitCFL=1.2, dtmin=1e-5, dtmax=3e-4),
    "C3": dict(nthm=1024, nzm=768, nrm=512, istr=6, str=20.0, ren=2e4, romeg=0.1, idtv=1, limitCFL=1.2,
               dtmin=1e-5, dtmax=1.8e-4),
    "C5": {},     # serving loop (run_serving)
}
DESCR = {
    "C2": "512x512x384 theta x z x r, wall-clustered radial grid ISTR=6 STR3=20, RINT=1 REXT=1.4, 1/NU=5000, "
          "AMPL_PERT=0.1 FREQ_PERT=0.5, RK3, variable dt CFLMAX=1.2 DTMIN=1e-5 DTMAX=3e-4, seeded Couette+noise 0.01",
    "C1": "64x64x64, ISTR=0, RINT=1 REXT=1.4, 1/NU=1000, RK3, dt=1e-3, seeded Couette+noise 0.01",
    "P2": "512x512x128 (profiling size of C2), ISTR=6 STR3=20, 1/NU=5000, RK3, variable dt",
    "C3": "1024x768x512, ISTR=6 STR3=20, ROTP=0.1, 1/NU=2e4, RK3, variable dt CFLMAX=1.2 DTMAX=1.8e-4 (FP64 form)",
    "C5": "serving loop",
}

# Algorithmic HBM bytes per cell and launch of each kernel class (FP64):
# the compulsory reads and writes of the arrays the kernel's job needs, each
# counted once (neighbour re-reads are not algorithmic).  P_SPEC is the
# fraction of a real field the half spectrum occupies: (nthm/2+1)/nthm complex.
def algorithmic_bytes(cls: str, nt: int, nz: int, nr: int, rk_substep_mix: float) -> float:
    cells = nt * nz * nr
    spec = (nt // 2 + 1) * 2 / nt          # complex doubles per cell, in doubles
    per_cell = {
        # read qt qr qz pr (+ ru1..3 on substeps with ro != 0), write rhs x3, ru x3
        "momentum": 8 * (4 + 3 * rk_substep_mix + 6),
        # read rhs x3 and q x3, write q x3
        "radial_solve": 8 * 9,
        # read qt qr qz, write half spectrum
        "div_theta_fft": 8 * (3 + spec),
        # read + write half spectrum
        "z_fft": 8 * 2 * spec,
        "pressure_tridiag": 8 * 2 * spec,
        # read half spectrum, write phi
        "theta_inverse_fft": 8 * (spec + 1),
        # read phi q x3 pr, write q x3 pr
        "correct": 8 * 9,
    }
    return per_cell.get(cls, 0.0) * cells


# Compulsory HBM bytes of one ideally fused RK3 step per cell: q (3 fields)
# read and written, pr read and written and one spectral round trip of phi per
# substep, plus the RK memory ru (read in substeps 2-3, written in 1-2).
# The FP64 fused momentum kernel (two cells a thread) measured by ncu on the
# 512x512x128 grid, one RK3 step (ncu --set full, one launch per substep): DRAM
# bytes per cell of a launch averaged over the three substeps (79.2, 102.9,
# 102.8), and per cell its FP64 instructions (45.41 DADD + 20.98 DMUL +
# 42.45 DFMA) and FLOPs.  Per-cell figures do not depend on the grid size.
MOMENTUM_FP64_NCU = {"dram_bytes_per_cell": 95.04, "fp64_inst_per_cell": 103.23, "fp64_flops_per_cell": 147.0}

STEP_BYTES = {"fp64": 3 * (6 + 2 + 2) * 8 + (2 * 3 + 2 * 3) * 8,
              "mixed": 3 * (6 * 4 + 2 * 8 + 2 * 4) + 12 * 4}


def base_bou(**kw):
    d = dict(nthm=64, nzm=64, nrm=64, nsst=3, idtv=1, nread=1, ntst=10 ** 8, tout=1.0e9, tmax=1.0e9,
             ireset=0, walltimemax=1e9, alx3=2 * math.pi, rint=1.0, rext=1.4, istr=0, str=4.0, lamb=1.0,
             virotint=1.0, virotext=0.0, sizepert=0.0, omegapert=0.0, ren=1000.0, romeg=0.0, resid=1e-2,
             limitCFL=1.2, tsta=0.0, starea=0, dtmin=1e-5, dtmax=1e-3, limitVel=1e3, cfllim=1.0,
             nslabr=0, dpthcut=0, dpstave=0, tframe2d=1.0, dpfullf=0, tframe3d=1.0,
             minstrt=0, minstrz=0, multmin=0)
    d.update(kw)
    return d


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_sample(workload: str, seconds: float, threads: int, nr_cap: int = 48):
    """Time the CPU oracle on a bounded sample of the workload: the same theta
    x z plane with the radial extent cut (to nr_cap cells) so one step takes a
    second or so."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import tc_ref
    import __graft_entry__ as entry
    entry.load()
    import tc_gb300.initial as ini
    tc_ref.build()
    tc_ref.set_threads(threads)
    w = dict(WORKLOADS[workload])
    nr_sample = min(w["nrm"], nr_cap)
    w["nrm"] = nr_sample
    bou = base_bou(**w)
    st = ini.couette_noise(bou, seed=1234)
    o = tc_ref.CppOracle(bou)
    o.set_state(*st)
    cells = bou["nthm"] * bou["nzm"] * bou["nrm"]
    o.run(0, 1, 0.0)                      # warm-up step (page faults, plans)
    n, t0 = 0, time.perf_counter()
    ntime, tsim = 1, 0.0
    while True:
        code, tsim, _ = o.run(ntime, 1, tsim)
        ntime += 1
        n += 1
        el = time.perf_counter() - t0
        if el > seconds or n >= 200:
            break
    return cells * n / el / 1e6, n, el, bou


def arm_config(workload: str, world: int) -> dict:
    """The `config` of the bench line; both arms print the same one."""
    w = WORKLOADS[workload]
    nt, nz, nr = w["nthm"], w["nzm"], w["nrm"]
    cells = nt * nz * nr
    return {"workload": f"{workload}: {DESCR[workload]}", "grid": [nt, nz, nr], "cells": cells,
            "precision": "FP64 plain", "parallelism": f"replicas x{world}",
            "l2": f"inputs larger than L2: every field is {cells * 8 / 1e6:.0f} MB, 12 fields resident"}


def run_reference(args, rank: int):
    """--impl reference: the CPU restatement of the reference's serial
    algorithm (the Fortran reference itself cannot be built: no Fortran
    compiler, MPI, FFTW or LAPACK here or on the GPU host) on every host
    core, on the full grid of the workload, one full RK3 step per step."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import tc_ref
    import __graft_entry__ as entry
    entry.load()
    import tc_gb300.initial as ini
    tc_ref.build()
    tc_ref.set_threads(threads)
    bou = base_bou(**WORKLOADS[args.workload])
    st = ini.couette_noise(bou, seed=1234)
    o = tc_ref.CppOracle(bou)
    o.set_state(*st)
    del st
    cells = bou["nthm"] * bou["nzm"] * bou["nrm"]
    ntime, tsim = 0, 0.0
    for _ in range(args.warmup):
        _, tsim, _ = o.run(ntime, 1, tsim)
        ntime += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, tsim, _ = o.run(ntime, 1, tsim)
        ntime += 1
    el = time.perf_counter() - t0
    v = cells * args.steps / el / 1e6
    sample = (f"the full {bou['nthm']}x{bou['nzm']}x{bou['nrm']} grid of the {args.workload} workload, "
              f"{args.steps} RK3 steps with the dt rule after {args.warmup} warm-up steps, C++ restatement "
              f"of the reference's serial algorithm, OpenMP on {threads} host cores")
    line = {"impl": "reference", "metric": "Mcell-steps/s", "value": v, "unit": "Mcell-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Couette+noise start)",
            "config": arm_config(args.workload, args.gpus),
            "cpu_baseline": {"value": v, "unit": "Mcell-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MATCHED_DT = ("one fixed dt per run in both forms: half the smallest dt the FP64 form's CFL rule picks over "
              "these steps after the DTMIN start steps")


def matched_torque_errors(tc, stream, bous, states, nsteps: int):
    """The mixed form's torque error alone, on the FP64 form's time grid.

    With its own dt rule each form picks dt from its own CFL number, and in
    the violent transient of a noisy start the two dt sequences part; so the
    FP64 form first runs the steps with its own rule, one at a time, to find
    each run's smallest dt after the DTMIN start steps, then both forms march
    with half of it, fixed (CFL <= 0.4 on that trajectory)."""
    ens = tc.Ensemble("fp64")
    ens.set_stream(stream.cuda_stream)
    sl = [ens.add(b, st, dt=0.0) for b, st in zip(bous, states)]
    dmin = [math.inf] * len(sl)
    for n in range(nsteps):
        ens.step(1)
        if n >= 2:
            for i, x in enumerate(sl):
                dmin[i] = min(dmin[i], ens.status_full(x)[2])
    ens.close()
    tq = {}
    for prec in ("fp64", "mixed"):
        ens = tc.Ensemble(prec)
        ens.set_stream(stream.cuda_stream)
        sl = [ens.add(b, st, dt=0.5 * d) for b, st, d in zip(bous, states, dmin)]
        ens.step(nsteps)
        tq[prec] = [ens.member(x).calc_torque() for x in sl]
        ens.close()
    return [max(abs(a[0] - b[0]) / abs(b[0]), abs(a[1] - b[1]) / abs(b[1])) for a, b in zip(tq["mixed"], tq["fp64"])]


def ensemble_legs(tc, torch, stream, steps: int, warmup: int, n_inst: int = 96, seed: int = 2024):
    """The batched-ensemble workload: n_inst instances with grids drawn from
    {32,48,64,96,128}^3, radius ratio in [0.5, 0.9], 1/NU log-uniform in
    [500, 5000], RK3 at CFL <= 0.8 (the reference's dt rule each step); FP64
    and mixed ensembles advanced by one CUDA graph per step, the schedule
    (grouped launches per phase, or one persistent launch per RK substep)
    and tile shape from the autotuner.  The mixed torque of every instance
    is compared with its FP64 torque after the same number of steps."""
    import tc_gb300.autotune as at
    import tc_gb300.initial as ini
    import tc_gb300.serving as sv
    bous = sv.draw_ensemble(n_inst, seed)
    states = [ini.couette_noise(b, seed=seed + i) for i, b in enumerate(bous)]
    out = {"instances": n_inst, "cells": int(sum(b["nthm"] * b["nzm"] * b["nrm"] for b in bous)),
           "grids": "drawn from {32,48,64,96,128}^3", "steps_timed": steps, "warmup": warmup}
    torques = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for prec in ("fp64", "mixed"):
        t0 = time.perf_counter()
        (thr, rows, sched, bps), table = at.tune(prec, bous, states, steps=2)
        tune_s = time.perf_counter() - t0
        ens = tc.Ensemble(prec)
        ens.set_stream(stream.cuda_stream)
        ens.tune(thr, rows, sched, bps)
        slots = [ens.add(b, st, nsteps=300, dt=0.0) for b, st in zip(bous, states)]
        ens.step(warmup)
        torch.cuda.synchronize()
        n0 = ens.launch_count
        e0.record(stream)
        ens.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        torques[prec] = [ens.member(sl).calc_torque() for sl in slots]
        codes = [ens.status_full(sl)[3] for sl in slots]
        out[prec] = {"value": out["cells"] * steps / (ms * 1e-3) / 1e6, "unit": "Mcell-steps/s",
                     "ms_per_step": ms / steps, "tile": {"threads": thr, "rows": rows, "schedule": sched, "blocks_per_sm": bps},
                     "best_ms_by_schedule": {s: round(min(v for k, v in table.items() if k.startswith(s)) * 1e3, 3)
                                             for s in ("grouped", "persistent")
                                             if any(k.startswith(s) for k in table)},
                     "tune_seconds": round(tune_s, 2), "tune_table_ms": {k: round(v * 1e3, 3) for k, v in
                                                                          table.items()},
                     "launches_per_step": ens.launches_per_step, "gpu_launches": ens.launch_count - n0,
                     "device_bytes": ens.device_bytes, "errorcodes_nonzero": sum(1 for c in codes if c)}
        ens.close()
    def rel(a, b):
        return max(abs(a[0] - b[0]) / abs(b[0]), abs(a[1] - b[1]) / abs(b[1]))

    errs = [rel(a, b) for a, b in zip(torques["mixed"], torques["fp64"])]
    out["torque_err_mixed_vs_fp64_own_dt"] = {
        "max": max(errs), "median": statistics.median(errs), "steps": warmup + steps,
        "note": "each form picks its own dt from its own CFL every step; in the violent transient of the "
                "noisy start the dt sequences part (dt swings 10x between steps), so this mixes the "
                "precision error with a different time grid"}
    nchk = warmup + steps
    errs = matched_torque_errors(tc, stream, bous, states, nchk)
    out["torque_err_mixed_vs_fp64"] = {"max": max(errs), "median": statistics.median(errs), "steps": nchk,
                                       "dt": MATCHED_DT}
    out["speedup_mixed_vs_fp64_ensemble"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def serving_leg(tc, torch, n: int, rates: list, chunk: int, hbm_budget: float, matched_runs: int = 6,
                with_clocks: bool = True) -> dict:
    """The serving workload: seeded Poisson arrivals swept over rates, runs of
    64^3 .. 256x256x128 cells and 100..2000 RK3 steps (variable dt, CFLMAX
    0.8), admitted against an HBM budget into one mixed-precision ensemble
    (continuous batching).  Beside it: the same runs one after another on
    the plain FP64 single-run path (tc_run), for the aggregate throughput
    and each run's torque."""
    import tc_gb300.autotune as at
    import tc_gb300.initial as ini
    import tc_gb300.serving as sv
    base = sv.draw_requests(n, rates[0], seed=7)
    states = {r.rid: ini.couette_noise(r.bou, seed=r.seed) for r in base}
    # sequential plain FP64 (the drop-in path), one run at a time
    seq_t0 = time.perf_counter()
    fp64_torque, fp64_cell_steps = {}, 0
    for r in base:
        g = tc.TaylorCouette(r.bou)
        g.set_state(*states[r.rid])
        code, _, _, _ = g.run(r.nsteps, 0, 0.0)
        fp64_torque[r.rid] = g.calc_torque()
        g.close()
        fp64_cell_steps += r.bou["nthm"] * r.bou["nzm"] * r.bou["nrm"] * r.nsteps
    seq_s = time.perf_counter() - seq_t0
    seq = {"value": fp64_cell_steps / seq_s / 1e6, "unit": "Mcell-steps/s", "wall_s": seq_s,
           "note": "same runs, one after another, tc_run on the plain FP64 path, host states in, torque out"}
    tile, _ = at.tune("mixed", [r.bou for r in base[:8]], [states[r.rid] for r in base[:8]], steps=2)
    sweep = []
    clocks = Clocks(0) if with_clocks else None
    for rate in rates:
        reqs = sv.with_rate(base, rate, seed=7)
        srv = sv.Server("mixed", hbm_budget=hbm_budget, chunk=chunk, tune=tile)
        res, stats = srv.run(reqs, lambda r: states[r.rid])
        lat = [x.latency for x in res]
        terr = []
        for x in res:
            w = fp64_torque[x.rid]
            terr.append(max(abs(x.torque[0] - w[0]) / abs(w[0]), abs(x.torque[1] - w[1]) / abs(w[1])))
        sweep.append({"rate_runs_per_s": rate, "requests": len(res), "p50_s": sv.percentile(lat, 0.5),
                      "p99_s": sv.percentile(lat, 0.99), "mean_s": sum(lat) / len(lat),
                      "value": stats["cell_steps"] / stats["wall_s"] / 1e6, "unit": "Mcell-steps/s",
                      "wall_s": stats["wall_s"], "peak_resident_runs": stats["peak_active"],
                      "peak_bytes": stats["peak_bytes"],
                      "torque_err_vs_fp64": {"max": max(terr), "median": statistics.median(terr)},
                      "errorcodes_nonzero": sum(1 for x in res if x.errorcode)})
    clk = clocks.stop() if clocks else None
    # precision error alone on the first runs, on the FP64 form's time grid
    mr = min(matched_runs, len(base))
    nchk = min(200, min(r.nsteps for r in base[:mr]))
    errs = matched_torque_errors(tc, torch.cuda.current_stream(), [r.bou for r in base[:mr]],
                                 [states[r.rid] for r in base[:mr]], nchk)
    matched = {"runs": mr, "steps": nchk, "max": max(errs), "median": statistics.median(errs), "dt": MATCHED_DT}
    best = max(sweep, key=lambda x: x["value"])
    return {"workload": "C5: serving loop, Poisson arrivals, grids 64^3..256x256x128, 100..2000 RK3 steps, "
                        "radius ratio 0.5..0.9, 1/NU 500..1e4, variable dt CFLMAX 0.8, "
                        f"{hbm_budget / 1e9:.0f} GB HBM budget, chunk {chunk} steps",
            "requests_per_rate": n, "tile": {"threads": tile[0], "rows": tile[1]},
            "serving": sweep, "best_value": best["value"], "sequential_fp64": seq,
            "torque_err_mixed_vs_fp64_matched_dt": matched,
            "torque_err_note": "torque_err_vs_fp64 in each sweep entry compares every served run at its end with "
                               "the FP64 run of the same request, each on its own CFL-driven dt sequence over up "
                               "to 2000 steps of a developing (at high Re, turbulent) flow; the matched-dt figure "
                               "isolates the precision error",
            "speedup_served_mixed_vs_sequential_fp64": best["value"] / seq["value"], "clocks": clk}


def run_serving(args):
    """--workload C5: the full serving sweep as its own bench line."""
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as entry
    tc = entry.load()
    import tc_gb300.build as tb
    tb.build()
    rates = [float(x) for x in args.rates.split(",")]
    leg = serving_leg(tc, torch, args.requests, rates, args.chunk, args.hbm_budget)
    line = {"metric": "Mcell-steps/s", "value": leg["best_value"], "unit": "Mcell-steps/s", "n_gpus": 1,
            "steps": None, "warmup": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/f64 mixed", "data": "synthetic (seeded Couette+noise starts, seeded Poisson arrivals)",
            "config": {"workload": leg["workload"], "requests_per_rate": args.requests, "tile": leg["tile"]},
            **{k: v for k, v in leg.items() if k not in ("workload", "tile", "requests_per_rate", "best_value")}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="C3", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed FP32/FP64 leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble legs")
    ap.add_argument("--ens-steps", type=int, default=20, help="timed steps of each ensemble leg")
    ap.add_argument("--ens-instances", type=int, default=96)
    ap.add_argument("--requests", type=int, default=16, help="C5: runs per arrival rate")
    ap.add_argument("--rates", default="0.5,1,2,5,10,20", help="C5: arrival rates, runs/s")
    ap.add_argument("--chunk", type=int, default=25, help="C5: steps between admissions")
    ap.add_argument("--hbm-budget", type=float, default=150e9)
    ap.add_argument("--no-serving", action="store_true", help="skip the short serving leg of the default run")
    ap.add_argument("--mixed-tma", action="store_true",
                    help="mixed legs: the TMA-staged momentum march instead of the cached one (the default)")
    ap.add_argument("--serve-requests", type=int, default=8, help="serving leg: runs per arrival rate")
    ap.add_argument("--serve-rates", default="2,20", help="serving leg: arrival rates, runs/s")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "C5":
        if rank == 0:
            run_serving(args)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import __graft_entry__ as entry
    tc = entry.load()
    import tc_gb300.build as tb
    tb.build()
    import tc_gb300.initial as ini

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    bou = base_bou(**WORKLOADS[args.workload])
    nt, nz, nr = bou["nthm"], bou["nzm"], bou["nrm"]
    cells = nt * nz * nr
    stream = torch.cuda.current_stream()
    g = tc.TaylorCouette(bou)
    g.set_stream(stream.cuda_stream)

    # seeded start in page-locked host memory on huge pages (reference layout)
    st = ini.couette_noise(bou, seed=1234 + rank)
    pinned = []
    for a in st:
        t = tc.host_array(a.shape)
        t[...] = a
        pinned.append(t)
    del st
    # host buffers of the same kind for the end-to-end run's result
    pinned_out = [tc.host_array(a.shape) for a in pinned]
    g.set_state(*pinned)

    # warm-up
    code, ntime, tsim, dt = g.run(args.warmup, 0, 0.0)
    if code != 0:
        raise SystemExit(f"warm-up stopped with error code {code}")

    # ---- device-resident timed region --------------------------------------
    clocks = Clocks(local) if rank == 0 else None
    g.profile(True)
    barrier()
    n0 = g.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    code, ntime, tsim, dt = g.run(args.steps, ntime, tsim)
    e1.record(stream)
    barrier()
    launches = g.launch_count - n0
    ms = max_over_ranks(e0.elapsed_time(e1))
    prof = g.profile_read()
    g.profile(False)
    clk = clocks.stop() if clocks else None
    if code != 0:
        raise SystemExit(f"timed steps stopped with error code {code}")
    value = world * cells * args.steps / (ms * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers ----------------------
    e2e = None
    if not args.no_e2e:
        # untimed warm-up of the same calls on the same host buffers (state in,
        # one step, state out), as the steps have theirs
        g.set_state(*pinned)
        g.run(1, 0, 0.0)
        g.get_state(out=pinned_out)
        barrier()
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.set_state(*pinned)
        ea.record(stream)
        nt2, t2 = 0, 0.0
        for _ in range(args.steps):
            code, nt2, t2, _ = g.run(1, nt2, t2)
        eb.record(stream)
        qt_o, qr_o, qz_o, pr_o = g.get_state(out=pinned_out)
        e1.record(stream)
        barrier()
        ms_e2e = max_over_ranks(e0.elapsed_time(e1))
        e2e_parts = {"set_state_ms": round(e0.elapsed_time(ea), 2), "steps_ms": round(ea.elapsed_time(eb), 2),
                     "get_state_ms": round(eb.elapsed_time(e1), 2)}
        h2d = sum(a.nbytes for a in pinned)
        d2h = h2d
        e2e = {"value": world * cells * args.steps / (ms_e2e * 1e-3) / 1e6, "unit": "Mcell-steps/s",
               "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
               "ms_per_step": ms_e2e / args.steps,
               "parts": e2e_parts,
               "note": "state in (tc_set_state) and out (tc_get_state) once per timed run, from and into "
                       "page-locked host buffers on huge pages (tc_host_alloc), amortised per step; dt/time "
                       "read back every step; one untimed "
                       "warm-up pass of the same calls on the same buffers before"}
        ref_state = tuple(a.copy() for a in (qt_o, qr_o, qz_o))
        ref_torque = g.calc_torque()

    # ---- the mixed FP32/FP64 forms on the same start ---------------------------
    # "mixed": FP64 pressure tridiagonals (the split of the specification);
    # "mixed-ff": the same with float-float pressure tridiagonals
    mixed = None
    if not args.no_mixed:
        forms = {}
        for prec in ("mixed", "mixed-ff"):
            gm = tc.TaylorCouette(bou, precision=prec)
            gm.set_stream(stream.cuda_stream)
            if args.mixed_tma:
                gm.use_tma(True)
            gm.set_state(*pinned)
            code_m, ntm, tm, _ = gm.run(args.warmup, 0, 0.0)
            gm.profile(True)
            barrier()
            e0.record(stream)
            code_m, ntm, tm, _ = gm.run(args.steps, ntm, tm)
            e1.record(stream)
            barrier()
            ms_m = max_over_ranks(e0.elapsed_time(e1))
            prof_m = gm.profile_read()
            gm.profile(False)
            leg = {"value": world * cells * args.steps / (ms_m * 1e-3) / 1e6, "unit": "Mcell-steps/s",
                   "ms_per_step": ms_m / args.steps, "speedup_vs_fp64": ms / ms_m, "status": code_m,
                   "pressure_tridiagonals": "FP64" if prec == "mixed" else "float-float",
                   "momentum_march": "TMA-staged" if args.mixed_tma else "cached"}
            tot_m = sum(v[0] for v in prof_m.values())
            leg["kernel_shares"] = {k: round(v[0] / tot_m, 4) for k, v in prof_m.items() if v[1]}
            leg["ms_per_step_by_kernel"] = {k: round(v[0] / args.steps, 3) for k, v in prof_m.items() if v[1]}
            if e2e is not None:
                gm.set_state(*pinned)
                gm.run(1, 0, 0.0)
                gm.get_state(out=pinned_out)
                barrier()
                e0.record(stream)
                gm.set_state(*pinned)
                nt3, t3 = 0, 0.0
                for _ in range(args.steps):
                    code_m, nt3, t3, _ = gm.run(1, nt3, t3)
                mstate = gm.get_state(out=pinned_out)
                e1.record(stream)
                barrier()
                ms_me = max_over_ranks(e0.elapsed_time(e1))
                leg["e2e"] = {"value": world * cells * args.steps / (ms_me * 1e-3) / 1e6, "unit": "Mcell-steps/s",
                              "ms_per_step": ms_me / args.steps}
                # error against the FP64 path after the same K steps from the same start
                errs = {}
                for name, a, b, nk in zip(("qt", "qr", "qz"), mstate[:3], ref_state, (nr, nr + 1, nr)):
                    a, b = a[1:-1, 1:-1, :nk], b[1:-1, 1:-1, :nk]
                    errs[name] = float(np.abs(a - b).max() / np.abs(b).max())
                ti, to = gm.calc_torque()
                errs["torque_inner"] = abs(ti - ref_torque[0]) / abs(ref_torque[0])
                errs["torque_outer"] = abs(to - ref_torque[1]) / abs(ref_torque[1])
                errs["max_divergence"] = gm.check_divergence()
                errs["steps"] = args.steps
                leg["err_vs_fp64"] = errs
            gm.close()
            forms[prec] = leg
        mixed = dict(forms["mixed"])
        mixed["float_float_pressure"] = forms["mixed-ff"]

    # ---- batched ensembles (FP64 and mixed) ----------------------------------
    ensemble = None
    if not args.no_ensemble:
        ensemble = ensemble_legs(tc, torch, stream, args.ens_steps, args.warmup, args.ens_instances)
        ensemble["speedup_mixed_ensemble_vs_plain_fp64"] = ensemble["mixed"]["value"] / value

    # ---- serving (continuous batching), a short sweep of two arrival rates ------
    serving = None
    if not args.no_serving and rank == 0:
        serving = serving_leg(tc, torch, args.serve_requests, [float(x) for x in args.serve_rates.split(",")],
                              args.chunk, args.hbm_budget, matched_runs=4, with_clocks=False)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel class ------------------------------
    peak_gbs, peak_kind = load_peaks()
    fp64_peak = g.measure_fp64_peak()
    dom = max((k for k in prof if k not in ("step_control", "reduction", "layout")), key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    rk_mix = 2.0 / 3.0   # ru read on 2 of the 3 RK3 substeps
    bytes_launch = algorithmic_bytes(dom, nt, nz, nr, rk_mix)
    achieved = bytes_launch / (dom_ms / dom_n * 1e-3) / 1e9
    traffic = None
    pipe = None
    if dom == "momentum":
        # DRAM bytes of a launch from the ncu capture, scaled by the cells;
        # the kernel's real limit is the FP64 pipe: its FP64 instruction rate
        # against the probe's (one DFMA = 2 FLOPs per instruction)
        traffic = MOMENTUM_FP64_NCU["dram_bytes_per_cell"] * cells
        t_launch = dom_ms / dom_n * 1e-3
        inst_rate = MOMENTUM_FP64_NCU["fp64_inst_per_cell"] * cells / t_launch
        peak_inst = fp64_peak * 1e12 / 2.0
        pipe = {"bound": "fp64 pipe", "unit": "FP64 instructions/s", "achieved": inst_rate, "peak": peak_inst,
                "frac": inst_rate / peak_inst,
                "fp64_tflops": MOMENTUM_FP64_NCU["fp64_flops_per_cell"] * cells / t_launch / 1e12,
                "peak_tflops": fp64_peak,
                "per_cell": {"fp64_instructions": MOMENTUM_FP64_NCU["fp64_inst_per_cell"],
                             "fp64_flops": MOMENTUM_FP64_NCU["fp64_flops_per_cell"]},
                "note": "per-cell FP64 instruction counts from ncu; peak = the FP64 FMA probe of this run"}
    total_ms = sum(v[0] for v in prof.values())
    shares = {k: round(v[0] / total_ms, 4) for k, v in prof.items() if v[1]}

    cpu = None
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, n, el, sb = cpu_sample(args.workload, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": "Mcell-steps/s", "cores": threads, "kind": "port",
               "sample": f"{n} steps of a {sb['nthm']}x{sb['nzm']}x{sb['nrm']} slab of the workload "
                         f"({el:.1f} s, C++ oracle, OpenMP on all host cores)"}
        # the same oracle on one core, on a thinner slab (serial baseline)
        v1, n1, el1, sb1 = cpu_sample(args.workload, min(args.cpu_seconds, 6.0), 1, nr_cap=8)
        cpu["serial"] = {"value": v1, "unit": "Mcell-steps/s", "cores": 1,
                         "sample": f"{n1} steps of a {sb1['nthm']}x{sb1['nzm']}x{sb1['nrm']} slab "
                                   f"({el1:.1f} s, C++ oracle, one thread)"}

    line = {
        "metric": "Mcell-steps/s", "value": value, "unit": "Mcell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Couette+noise start)",
        "config": arm_config(args.workload, world),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                     "frac": achieved / peak_gbs, "peak_kind": f"{peak_kind} hbm_gbs",
                     "traffic": traffic, "algorithmic_bytes_per_launch": bytes_launch,
                     "ms_per_launch": dom_ms / dom_n, "launches": dom_n,
                     "traffic_note": "ncu DRAM bytes per cell on the 512x512x128 grid x cells" if traffic else None,
                     "compute": pipe},
        "step_roofline": {
            "bytes_per_cell_step": STEP_BYTES["fp64"], "achieved": value * 1e6 * STEP_BYTES["fp64"] / 1e9,
            "peak": peak_gbs, "unit": "GB/s", "frac": value * 1e6 * STEP_BYTES["fp64"] / 1e9 / peak_gbs,
            "mixed_frac": (mixed["value"] * 1e6 * STEP_BYTES["mixed"] / 1e9 / peak_gbs) if mixed else None,
            "note": "whole RK3 step against the compulsory state traffic of an ideally fused step "
                    "(336 B/cell-step FP64, 192 mixed)"},
        "fp64": {"probe_tflops": fp64_peak,
                 "note": "FP64 FMA rate of the device measured by a probe kernel; the FP64 path is "
                         "bounded by it rather than by HBM"},
        "kernel_shares": shares,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "mixed": mixed,
        "ensemble": ensemble,
        "serving": serving,
        "gpu_launches": launches,
        "clocks": clk,
        "sim": {"time": tsim, "last_dt": dt},
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

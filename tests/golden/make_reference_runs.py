"""Golden fixtures from runs of the reference's own Fortran source.

The reference's main program (main.F90, `papero`) and every routine of its
time step are executed by tests/golden/fortran_subset.py (a translator of
the Fortran subset they use, with a one-rank runtime of MPI, 2DECOMP&FFT,
FFTW, HDF5 and LAPACK; LAPACK is SciPy's).  Each case writes its bou.in,
starts from a seeded Couette-plus-noise field read through the NREAD=1
continua path (pressure zero), and runs until the reference's QuitRoutine
(error code 555 after NTST+1 steps, or an earlier stop).  Recorded per case:

* the final qt, qr, qz, pr in the reference layout (nthm+2, nzm+2, nr)
  in C order, i.e. Fortran q(1:nr, 0:nzm+1, 0:nthm+1), halos included;
* per step: time and dt after the step, and the CFL number of the
  CalcMaxCFL call at the top of the step (the one its dt rule used);
* per output step (main.F90: ntime = 1 or mod(time, tout) < dt): the
  CalcTorque record (time, inner, outer) and vmax of CalcVelocityStats
  and its rms_vel.out record (time, qt, qr, qz rms);
  the CheckDivergence maxima (the first one is the check before the loop);
* the error code and ntime of the stop;
* after the stop: CalcTorque, CheckDivergence and CalcMaxCFL of the final
  state, called directly;
* the 1-D grid and coefficient arrays of CreateGrid and InitPressureSolver;
* where a case asks for them: the statistics accumulations, sample count
  and dissipation records; every HDF5 file the run wrote (dumps, and
  WriteStats / WriteFlowField / WriteGridInfo) and the files it was given;
  what every routine of the first step's substeps wrote; the start that
  CreateInitialConditions (NREAD = 0) or ReadFlowField's interpolation from
  another grid built.

Usage (needs the reference tree; SciPy for LAPACK):

    python tests/golden/make_reference_runs.py [--ref /root/reference] [--only NAME]

writes tests/golden/reference_runs.npz and reference_runs.json (the cases,
their bou values and seeds).  The fixtures are committed; the tests read
them and never need the reference tree.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "taylor-couette-afid_gb300"))

import fortran_subset as fs  # noqa: E402
import initial as ini  # noqa: E402

# the time-step path of the reference and what main.F90 calls around it
FILES = ["main.F90", "ReadInputFile.F90", "InitTimeMarchScheme.F90", "InitVariables.F90", "CreateGrid.F90",
         "InitPressureSolver.F90", "ReadFlowField.F90", "CheckDivergence.F90", "CalcMaxCFL.F90", "TimeMarcher.F90",
         "InnerCylVelocity.F90", "SlipBCs.F90", "ExplicitTermsQT.F90", "ExplicitTermsQR.F90", "ExplicitTermsQZ.F90",
         "ImplicitAndUpdateQT.F90", "ImplicitAndUpdateQR.F90", "ImplicitAndUpdateQZ.F90",
         "SolveImpEqnUpdate_QT.F90", "SolveImpEqnUpdate_QR.F90", "SolveImpEqnUpdate_QZ.F90",
         "CalcLocalDivergence.F90", "SolvePressureCorrection.F90", "CorrectVelocity.F90", "CorrectPressure.F90",
         "CalcVelocityStats.F90", "CalcTorque.F90", "AuxiliaryRoutines.F90", "StatRoutines.F90",
         "CalcVorticity.F90", "CalcDissipation.F90", "interp.F90", "StatReadReduceWrite.F90", "WriteFlowField.F90",
         "DumpRCuts.F90", "DumpThCuts.F90", "DumpStreamwiseAvg.F90", "DumpFlowField.F90", "WriteGridInfo.F90",
         "CreateInitialConditions.F90"]
# the 1-D arrays of CreateGrid and InitPressureSolver (module param)
GRID_NAMES = ["rc", "rm", "g2rc", "g2rm", "usrc", "usrm", "udx1vis1", "udx1vis2", "udx1qm", "udx2c", "udx2m",
              "rudx2c", "udx2rm", "ap1j", "am1j", "ac1j", "ap2j", "am2j", "ac2j", "ap2je", "am2je", "ac2je", "ap3j",
              "am3j", "ac3j", "apph", "amph", "acph", "pvol", "udx2mm", "udx2cc", "ak1", "ak3"]
STAT_NAMES = ["vt_me", "vr_me", "vz_me", "wt_me", "wr_me", "wz_me", "vt_rms", "vr_rms", "vz_rms", "wt_rms", "wr_rms",
              "wz_rms", "vtvr_me", "vtvz_me", "vrvz_me", "pr_me", "pr_rms", "disste"]
MODULE_FILES = ["param.F90"]

BOU_ORDER = [
    ("NTM  NZM  NRM  NSST  IDTV    NREAD", ["nthm", "nzm", "nrm", "nsst", "idtv", "nread"]),
    ("NTST      TOUT      TMAX     IRESET    WALLTIMEMAX(s)", ["ntst", "tout", "tmax", "ireset", "walltimemax"]),
    ("ALX3D    RINT    REXT  ISTR   STR3    LAMB", ["alx3", "rint", "rext", "istr", "str", "lamb"]),
    ("VIROTINT VIROTEXT   AMPL_PERT   FREQ_PERT", ["virotint", "virotext", "sizepert", "omegapert"]),
    ("1/NU       ROTP    RESID    CFLMAX", ["ren", "romeg", "resid", "limitCFL"]),
    ("TSTA  STAREAD", ["tsta", "starea"]),
    ("DTMIN    DTMAX  VMAX     CFLLIM(dt fixed)", ["dtmin", "dtmax", "limitVel", "cfllim"]),
    ("NOUT_RCUT  OUT_THCUT  OUT_STWAVE   TFRAME2D", ["nslabr", "dpthcut", "dpstave", "tframe2d"]),
    ("OUT_3DFIELD TFRAME3D", ["dpfullf", "tframe3d"]),
    ("MINSTRT (Nx)      MINSTRZ (Nz)     MULTMIN (Nf)", ["minstrt", "minstrz", "multmin"]),
]
INTS = {"nthm", "nzm", "nrm", "nsst", "idtv", "nread", "ntst", "ireset", "istr", "starea", "nslabr", "dpthcut",
        "dpstave", "dpfullf", "minstrt", "minstrz", "multmin"}


def bou_text(bou):
    """bou.in in the reference's layout (a header line before each record);
    reals in repr form, which list-directed input reads exactly."""
    out = []
    for head, keys in BOU_ORDER:
        out.append(" " + head)
        vals = []
        for k in keys:
            v = bou[k]
            vals.append(str(int(v)) if k in INTS else repr(float(v)))
        out.append("  " + "   ".join(vals))
    return "\n".join(out) + "\n"


def base_bou(**kw):
    d = dict(nthm=16, nzm=12, nrm=10, nsst=3, idtv=1, nread=1, ntst=19, tout=1.0e6, tmax=1.0e6, ireset=0,
             walltimemax=1e9, alx3=2 * math.pi, rint=1.0, rext=1.4, istr=0, str=4.0, lamb=1.0, virotint=1.0,
             virotext=0.0, sizepert=0.0, omegapert=0.0, ren=1000.0, romeg=0.0, resid=1e-2, limitCFL=1e3,
             tsta=1.0e9, starea=0, dtmin=1e-3, dtmax=1e-3, limitVel=1e3, cfllim=1.0, nslabr=0, dpthcut=0,
             dpstave=0, tframe2d=1.0, dpfullf=0, tframe3d=1.0, minstrt=0, minstrz=0, multmin=0)
    d.update(kw)
    return d


# Cases: each covers a part of the path the GPU parity tests also cover.
CASES = [
    dict(name="uniform_rk3_fixed_dt", seed=11, amp=0.01,
         bou=base_bou()),
    dict(name="tanh_rk3_variable_dt_oscillating", seed=12, amp=0.01,
         bou=base_bou(nthm=12, nzm=16, nrm=12, istr=4, str=1.5, idtv=1, limitCFL=1.2, dtmin=1e-5, dtmax=2e-3,
                      sizepert=0.1, omegapert=0.5, ren=800.0, tout=4e-3)),
    dict(name="chebyshev_rk3_rotating", seed=13, amp=0.02,
         bou=base_bou(nthm=16, nzm=10, nrm=12, istr=6, str=3.0, romeg=0.1, ren=2.0e4, idtv=1, limitCFL=1.2,
                      dtmin=1e-5, dtmax=1.8e-3, tout=5e-3)),
    dict(name="uniform_ab2", seed=14, amp=0.01,
         bou=base_bou(nthm=12, nzm=12, nrm=8, nsst=1, dtmin=5e-4, dtmax=5e-4)),
    # AB2 with the dt rule: the multistep weights stay those of a constant
    # step while dt changes (InitTimeMarchScheme.F90)
    dict(name="ab2_variable_dt_tanh", seed=29, amp=0.03,
         bou=base_bou(nthm=16, nzm=12, nrm=10, nsst=1, istr=4, str=2.0, idtv=1, limitCFL=0.4, dtmin=1e-4,
                      dtmax=2e-3, ntst=14, tout=3e-3)),
    # patterned slip on the oscillating, rotating inner cylinder over many
    # steps (the slip pattern moves with the wall, SlipBCs.F90)
    dict(name="patterned_slip_oscillating_rotating", seed=30, amp=0.02,
         bou=base_bou(nthm=16, nzm=16, nrm=8, minstrt=2, minstrz=2, multmin=1, rext=1.5, alx3=2.0, istr=6,
                      str=3.0, sizepert=0.15, omegapert=2.0, romeg=0.1, ntst=14, dtmin=2e-3, dtmax=2e-3,
                      tout=6e-3)),
    dict(name="patterned_slip", seed=15, amp=0.01,
         bou=base_bou(nthm=16, nzm=16, nrm=8, minstrt=2, minstrz=2, multmin=1, ntst=9, virotint=1.0,
                      rext=1.5, lamb=1.0, alx3=2.0)),
    dict(name="aspect_lamb_virotext", seed=16, amp=0.03,
         bou=base_bou(nthm=10, nzm=10, nrm=9, istr=6, str=2.0, lamb=3.0, alx3=1.7, rint=0.8, rext=1.3,
                      virotext=0.3, virotint=0.9, idtv=1, limitCFL=0.9, dtmin=1e-5, dtmax=3e-3, tout=1e-2)),
    dict(name="stops_at_tmax", seed=17, amp=0.01,
         bou=base_bou(nthm=8, nzm=8, nrm=6, tmax=4.5e-3, ntst=100)),
    dict(name="dt_below_dtmin", seed=18, amp=0.01,
         bou=base_bou(nthm=8, nzm=8, nrm=6, idtv=1, limitCFL=1e-4, dtmin=1e-3, dtmax=2e-3, ntst=10)),
    dict(name="output_every_step", seed=19, amp=0.05,
         bou=base_bou(nthm=12, nzm=10, nrm=10, istr=6, str=5.0, tout=1e-3, ntst=14)),
    # transform lengths with the prime factors 7, 13 (theta 14 -> 7 complex
    # points, z 26) and 11 (theta 22, z 22)
    dict(name="prime_lengths_7_13", seed=20, amp=0.02,
         bou=base_bou(nthm=14, nzm=26, nrm=8, istr=6, str=3.0, ntst=9)),
    dict(name="prime_lengths_11", seed=21, amp=0.02,
         bou=base_bou(nthm=22, nzm=22, nrm=7, ntst=9, idtv=1, limitCFL=1.0, dtmin=1e-5, dtmax=2e-3)),
    # the production case (512x512x384, ISTR=6, STR3=20, 1/NU=5000,
    # oscillating inner cylinder, CFLMAX 1.2, DTMAX 3e-4) on a smaller grid
    dict(name="production_oscillating_32x24x32", seed=1234, amp=0.01,
         bou=base_bou(nthm=32, nzm=24, nrm=32, istr=6, str=20.0, ren=5000.0, sizepert=0.1, omegapert=0.5,
                      idtv=1, limitCFL=1.2, dtmin=1e-5, dtmax=3e-4, tout=2e-3)),
    # the rotating case (1024x768x512, ROTP=0.1, 1/NU=2e4, DTMAX 1.8e-4)
    # on a smaller grid
    dict(name="rotating_32x24x32", seed=4321, amp=0.01,
         bou=base_bou(nthm=32, nzm=24, nrm=32, istr=6, str=20.0, ren=2.0e4, romeg=0.1, idtv=1, limitCFL=1.2,
                      dtmin=1e-5, dtmax=1.8e-4, tout=1e-3)),
    # the CPU-runnable case at its own size: 64^3, ISTR=0, 1/NU=1000, dt 1e-3
    # (fixed through IDTV=1, DTMIN = DTMAX), the first 5 steps; fields
    # kept on four theta planes plus whole-field sums
    dict(name="c1_64cubed_5_steps", seed=2024, amp=0.01, planes=[1, 17, 33, 64],
         bou=base_bou(nthm=64, nzm=64, nrm=64, ntst=4)),
    # the parameters of the 1024x768x512 benchmark (wall-clustered grid
    # ISTR=6 STR3=20, ROTP=0.1, 1/NU=2e4, variable dt with CFLMAX=1.2 and
    # DTMAX=1.8e-4) on a 128x96x64 grid, 5 steps; some theta planes kept
    dict(name="c3_parameters_128x96x64_5_steps", seed=1234, amp=0.01, planes=[1, 33, 65, 128],
         bou=base_bou(nthm=128, nzm=96, nrm=64, istr=6, str=20.0, ren=2e4, romeg=0.1, idtv=1, limitCFL=1.2,
                      dtmin=1e-5, dtmax=1.8e-4, ntst=4)),
    # the parameters of the 512x512x384 production case (ISTR=6 STR3=20,
    # 1/NU=5000, the oscillating inner cylinder, DTMAX=3e-4) on 96x128x48
    dict(name="c2_parameters_96x128x48_5_steps", seed=1234, amp=0.01, planes=[1, 25, 49, 96],
         bou=base_bou(nthm=96, nzm=128, nrm=48, istr=6, str=20.0, ren=5000.0, sizepert=0.1, omegapert=0.5,
                      idtv=1, limitCFL=1.2, dtmin=1e-5, dtmax=3e-4, ntst=4)),
    # statistics on (TSTA = 0): main.F90 calls CalcStats (with
    # CalcVorticity) and CalcDissipation at every output step
    # statistics every output step, radial/theta/streamwise-average slabs
    # every other one, full-field dumps every third; the files the run
    # writes (dumps, WriteStats and WriteFlowField at the stop) are kept
    dict(name="statistics_and_dumps", seed=22, amp=0.05, stats=True, files=True, rcuts=[1.05, 1.23],
         bou=base_bou(nthm=16, nzm=12, nrm=10, istr=6, str=3.0, romeg=0.15, tsta=0.0, tout=2e-3, ntst=9,
                      nslabr=2, dpthcut=1, dpstave=1, tframe2d=4e-3, dpfullf=1, tframe3d=6e-3)),
    # a restart whose continua files hold time 1.2345: the run goes on from
    # that time (the oscillating wall's phase, the output steps) and TMAX
    # counts from it (stop 333 after time 1.2345 + 0.0601)
    dict(name="restart_at_a_later_time", seed=27, amp=0.03, start_time=1.2345,
         bou=base_bou(nthm=12, nzm=10, nrm=8, istr=4, str=1.5, sizepert=0.2, omegapert=0.7, tout=3e-3,
                      tmax=0.0601, ntst=100)),
    # one step on a tanh grid with rotation, the oscillating wall (from time
    # 0.37) and patterned slip: every routine's output of its three
    # substeps is kept
    dict(name="routine_outputs_of_one_step", seed=28, amp=0.05, start_time=0.37, routines=True,
         bou=base_bou(nthm=16, nzm=16, nrm=8, istr=4, str=2.0, romeg=0.1, sizepert=0.1, omegapert=0.5,
                      minstrt=2, minstrz=2, multmin=1, ntst=0, rext=1.5, alx3=2.0)),
    # stops at the first output step: velocities above VMAX (266), and the
    # divergence above RESID (169)
    dict(name="velocities_above_vmax", seed=25, amp=0.05,
         bou=base_bou(nthm=12, nzm=10, nrm=8, limitVel=4e-3)),
    dict(name="divergence_above_resid", seed=26, amp=0.05,
         bou=base_bou(nthm=12, nzm=10, nrm=8, resid=1e-30)),
    # STAREAD = 1: statistics files of an earlier run are read and added to
    # this run's at the stop (StatReadReduceWrite)
    dict(name="statistics_read_and_added", seed=24, amp=0.05, stats=True, files=True, stats_in=7,
         bou=base_bou(nthm=12, nzm=10, nrm=8, istr=4, str=2.0, tsta=0.0, tout=3e-3, ntst=7, starea=1)),
    # the reference's own initial condition (NREAD = 0: CreateInitialConditions)
    dict(name="created_initial_conditions", seed=0, amp=0.0,
         bou=base_bou(nthm=16, nzm=12, nrm=10, nread=0, istr=4, str=2.0, ren=800.0, ntst=14, tout=4e-3,
                      dtmin=1e-4, dtmax=1e-2, limitCFL=2e-3)),
    # a restart from continua files of a coarser grid: ReadFlowField
    # interpolates them (interp.F90) onto the run's grid; the start is kept
    dict(name="restart_interpolated_from_coarser_grid", seed=23, amp=0.05,
         old_grid=dict(nthm=8, nzm=8, nrm=6),
         bou=base_bou(nthm=12, nzm=14, nrm=9, istr=0, ntst=4)),
]


class _Started(Exception):
    """Raised after ReadFlowField in the restart cases: only the start is kept."""


def run_restart(ref_dir, case):
    """The interpolated start of a restart from a coarser grid, twice: with
    undefined values as NaN (the mask of points that depend on memory the
    reference never sets: interp.F90 reads corner halos of the old field
    that nothing fills) and as zeros (the values)."""
    out = {}
    for nan_fill in (True, False):
        try:
            run_case(ref_dir, case, stop_after_read=True, nan_fill=nan_fill)
        except _Started as st:
            for k, a in st.args[0].items():
                if nan_fill:
                    out["start_defined_" + k] = np.isfinite(a)
                else:
                    out["start_" + k] = a
    return out


def run_case(ref_dir, case, verbose=False, stop_after_read=False, nan_fill=True):
    if case.get("old_grid") and not stop_after_read:
        return run_restart(ref_dir, case)
    bou = dict(case["bou"])
    qt, qr, qz, pr = ini.couette_noise(bou, seed=case["seed"], amp=case["amp"])
    nrm = int(bou["nrm"])
    nr = nrm + 1
    nth, nz = int(bou["nthm"]) + 1, int(bou["nzm"]) + 1

    def interior(a):   # (nthm+2, nzm+2, nr) C order -> Fortran (nr, nzm, nthm)
        return np.asfortranarray(a[1:-1, 1:-1, :].transpose(2, 1, 0))

    continua = {"qt": interior(qt), "qr": interior(qr), "qz": interior(qz), "nth": nth, "nr": nr, "nz": nz,
                "time": float(case.get("start_time", 0.0)), "istr": int(bou["istr"]), "str": float(bou["str"])}
    if case.get("old_grid"):
        # the continua files hold the same seeded start on a coarser grid
        obou = dict(bou, **case["old_grid"])
        oq = ini.couette_noise(obou, seed=case["seed"], amp=case["amp"])
        continua.update(qt=interior(oq[0]), qr=interior(oq[1]), qz=interior(oq[2]), nth=int(obou["nthm"]) + 1,
                        nr=int(obou["nrm"]) + 1, nz=int(obou["nzm"]) + 1)
    files = {"bou.in": bou_text(bou), "continua_master.h5": ""}
    if case.get("rcuts"):
        # rcuts.in: a header record, then the radii of the slabs (InitDumpRCuts)
        files["rcuts.in"] = " RCUT\n  " + "   ".join(repr(float(r)) for r in case["rcuts"]) + "\n"
    rt = fs.OneRank(files, continua)
    h5_in = stats_files_in(bou, case["stats_in"]) if case.get("stats_in") is not None else {}
    for fname, dsets in h5_in.items():
        rt.h5[fname] = {k: v.copy() for k, v in dsets.items()}
    w = fs.World(ref_dir, FILES, MODULE_FILES, rt, capture_units=(97, 92, 98), nan_fill=nan_fill)
    F, G = w.F, w.G
    start = {}
    orig_read = F.readflowfield

    def readflowfield(*a):
        r = orig_read(*a)
        for k in ("qt", "qr", "qz"):
            start[k] = np.ascontiguousarray(getattr(G, k).d.transpose(2, 1, 0)).copy()
        if stop_after_read:
            raise _Started(start)
        return r

    F.readflowfield = readflowfield
    orig_create = F.createinitialconditions

    def createinitialconditions(*a):
        r = orig_create(*a)
        for k in ("qt", "qr", "qz"):
            start[k] = np.ascontiguousarray(getattr(G, k).d.transpose(2, 1, 0)).copy()
        return r

    F.createinitialconditions = createinitialconditions
    orig_ws = F.writestats
    samples = []

    def writestats(*a):
        # the run's own sample count (WriteStats adds a read file's to it)
        samples.append(int(G.nstatsamples))
        return orig_ws(*a)

    F.writestats = writestats
    rec = {"cfl": [], "time": [], "dt": [], "dmax": [], "vmax": [], "step_cfl": []}
    orig = {n: getattr(F, n) for n in ("timemarcher", "calcmaxcfl", "checkdivergence", "calcvelocitystats")}

    def timemarcher(*a):
        # the CFL number the dt rule of this step used: the last CalcMaxCFL
        # (main.F90 calls it at the top of every step)
        rec["step_cfl"].append(rec["cfl"][-1])
        r = orig["timemarcher"](*a)
        rec["time"].append(G.time + G.dt)
        rec["dt"].append(G.dt)
        if verbose:
            print(f"  step ntime={G.ntime} dt={G.dt:.6e}", flush=True)
        return r

    def calcmaxcfl(c):
        r = orig["calcmaxcfl"](c)
        rec["cfl"].append(float(r[0]))
        return r

    def checkdivergence(q):
        r = orig["checkdivergence"](q)
        rec["dmax"].append(float(r[0]))
        return r

    def calcvelocitystats(*a):
        r = orig["calcvelocitystats"](*a)
        rec["vmax"].append([float(x) for x in G.vmax.d])
        return r

    F.timemarcher, F.calcmaxcfl, F.checkdivergence, F.calcvelocitystats = (
        timemarcher, calcmaxcfl, checkdivergence, calcvelocitystats)
    routines = {}
    if case.get("routines"):
        # what every routine of the first step's substeps leaves in the
        # arrays it writes (TimeMarcher.F90:31-54), C order
        writes = {"explicittermsqt": ("dq",), "explicittermsqr": ("dph",), "explicittermsqz": ("qcap",),
                  "implicitandupdateqt": ("qt", "ru1"), "implicitandupdateqr": ("qr", "ru2"),
                  "implicitandupdateqz": ("qz", "ru3"), "calclocaldivergence": ("dph",),
                  "solvepressurecorrection": ("dph",), "correctvelocity": ("qt", "qr", "qz"),
                  "correctpressure": ("pr",)}
        counts = {}

        def recorder(name, fn):
            def wrapped(*a):
                r = fn(*a)
                if not rec["time"]:            # inside the first TimeMarcher
                    ns = counts[name] = counts.get(name, 0) + 1
                    for arr in writes[name]:
                        routines[f"routine:{ns}:{name}:{arr}"] = np.ascontiguousarray(
                            getattr(G, arr).d.transpose(2, 1, 0)).copy()
                return r
            return wrapped

        for name in writes:
            setattr(F, name, recorder(name, getattr(F, name)))
    t0 = time.time()
    code = None
    try:
        F.papero()
    except fs.Quit as q:
        code = q.errorcode
    torques_out = [list(map(float, r)) for r in rt.written.get(97, [])]
    nutes = [list(map(float, r)) for r in rt.written.get(92, [])]
    stats = {n: np.ascontiguousarray(getattr(G, n).d.T) for n in STAT_NAMES} if case.get("stats") else {}
    nsamples = samples[0] if samples else int(G.nstatsamples)
    F.checkdivergence, F.calcmaxcfl = orig["checkdivergence"], orig["calcmaxcfl"]
    final_dmax = float(F.checkdivergence(0.0)[0])
    final_cfl = float(F.calcmaxcfl(0.0)[0])
    F.calctorque()
    final_torque = [float(x) for x in rt.written[97][-1]]

    def state(a):   # Fortran (nr, nzm+2, nthm+2) -> C order (nthm+2, nzm+2, nr)
        return np.ascontiguousarray(a.d.transpose(2, 1, 0))

    fields = dict(qt=state(G.qt), qr=state(G.qr), qz=state(G.qz), pr=state(G.pr))
    for k, v in fields.items():
        if not np.all(np.isfinite(v)):
            raise RuntimeError(f"{case['name']}: {k} is not finite")
    out = {}
    planes = case.get("planes")
    for k, v in fields.items():
        if planes is None:
            out[k] = v
        else:
            out[k + "_planes"] = np.ascontiguousarray(v[planes])
            out.update(field_sums(k, v))
    out.update(dict(step_time=np.array(rec["time"]), step_dt=np.array(rec["dt"]), step_cfl=np.array(rec["step_cfl"]),
               out_torque=np.array(torques_out).reshape(-1, 3), out_dmax=np.array(rec["dmax"]),
               out_vmax=np.array(rec["vmax"]).reshape(-1, 3),
               out_rms=np.array([list(map(float, r)) for r in rt.written.get(98, [])]).reshape(-1, 4), errorcode=np.array(code), ntime=np.array(G.ntime),
               final_time=np.array(G.time), final_dmax=np.array(final_dmax), final_cfl=np.array(final_cfl),
               final_torque=np.array(final_torque)))
    if int(bou["nread"]) == 0:
        # the reference's own start (before the halo update of main.F90:120)
        for k, a in start.items():
            out["start_" + k] = a
    out.update(routines)
    for n in GRID_NAMES:
        out["grid_" + n] = np.array(getattr(G, n).d, dtype=np.float64).reshape(-1).copy()
    for fname, dsets in sorted(h5_in.items()):
        for dname, a in dsets.items():
            out[f"h5in:{fname}:{dname}"] = a
    if case.get("files"):
        for fname, dsets in sorted(rt.h5.items()):
            for dname, a in dsets.items():
                out[f"h5:{fname}:{dname}"] = a
    if case.get("stats"):
        out["stat_samples"] = np.array(nsamples)
        out["out_nute"] = np.array(nutes).reshape(-1, 2)
        for n, a in stats.items():
            out["stat_" + n] = a

    if verbose:
        print(f"{case['name']}: code {code}, ntime {G.ntime}, {len(rec['dt'])} steps, {time.time() - t0:.1f} s")
    return out


STAT_FILES = ["vt_mean", "vr_mean", "vz_mean", "wt_mean", "wr_mean", "wz_mean", "vt_rms", "vr_rms", "vz_rms",
              "wt_rms", "wr_rms", "wz_rms", "vtvr_mean", "vtvz_mean", "vrvz_mean", "pr_mean", "pr_rms", "disste"]


def stats_files_in(bou, seed):
    """Statistics files of an earlier run (stats/<name>.h5 with dataset
    <name>, C order (nzm, nrm); stats/stafield_master.h5 with its sample
    count): seeded values."""
    nzm, nrm = int(bou["nzm"]), int(bou["nrm"])
    out = {"stats/stafield_master.h5": {"averaging_time": np.array([3], dtype=np.int32)}}
    for i, n in enumerate(STAT_FILES):
        out[f"stats/{n}.h5"] = {n: ini.uniform(seed, 10 + i, 1, nzm, nrm)[0]}
    return out


def field_sums(k, v):
    """Whole-field checks kept when a case stores only some planes: the sum,
    the sum of squares and a sum weighted by a fixed pseudo-random pattern
    over the interior cells (pressure with its radial profile removed)."""
    a = v[1:-1, 1:-1, :]
    if k == "pr":
        a = a[..., :-1]
        a = a - a.mean(axis=(0, 1), keepdims=True)
    w = ini.uniform(99, 7, a.shape[0], a.shape[1], a.shape[2])
    return {k + "_sum": np.array(a.sum()), k + "_sumsq": np.array((a * a).sum()),
            k + "_wsum": np.array((a * w).sum())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default=None)
    ap.add_argument("--out", default=os.path.join(HERE, "reference_runs"))
    ap.add_argument("-v", action="store_true")
    args = ap.parse_args()
    arrays, meta = {}, []
    old = {}
    if args.only and os.path.exists(args.out + ".npz"):
        with np.load(args.out + ".npz") as z:
            old = {k: z[k] for k in z.files}
        with open(args.out + ".json") as f:
            meta = [m for m in json.load(f)["cases"] if m["name"] != args.only]
    # keep the other cases of the committed fixture (no stale keys of cases
    # that are gone or of the case being rerun)
    names = [c["name"] for c in CASES]
    arrays.update({k: v for k, v in old.items() if k.split("/")[0] in names and k.split("/")[0] != args.only})
    meta = [m for m in meta if m["name"] in names]
    for case in CASES:
        if args.only and case["name"] != args.only:
            continue
        res = run_case(args.ref, case, verbose=args.v)
        for k, v in res.items():
            arrays[f"{case['name']}/{k}"] = v
        meta = [m for m in meta if m["name"] != case["name"]]
        meta.append(dict(name=case["name"], seed=case["seed"], amp=case["amp"], bou=case["bou"],
                         planes=case.get("planes"), stats=bool(case.get("stats")),
                         files=bool(case.get("files")), rcuts=case.get("rcuts"), old_grid=case.get("old_grid"),
                         stats_in=case.get("stats_in"), start_time=case.get("start_time", 0.0)))
    order = [c["name"] for c in CASES]
    meta.sort(key=lambda m: order.index(m["name"]))
    np.savez_compressed(args.out + ".npz", **arrays)
    sources = {}
    for fn in MODULE_FILES + FILES:
        with open(os.path.join(args.ref, fn), "rb") as f:
            sources[fn] = hashlib.sha256(f.read()).hexdigest()
    with open(args.out + ".json", "w") as f:
        json.dump({"generator": "tests/golden/make_reference_runs.py", "executed_sources_sha256": sources,
                   "cases": meta}, f, indent=1)
    print(f"wrote {args.out}.npz ({os.path.getsize(args.out + '.npz') / 1e3:.0f} kB), {len(meta)} cases")


if __name__ == "__main__":
    main()

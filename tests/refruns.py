"""The golden runs of the reference's own Fortran source and how a
simulation is compared with them.

tests/golden/reference_runs.npz / .json hold runs of the reference's main
program (main.F90 and every routine of its time step, executed on one rank
by tests/golden/fortran_subset.py; see tests/golden/make_reference_runs.py):
for each case its bou.in values and seed, the final fields, the dt sequence,
the CFL number behind each dt, the CalcTorque records of the output steps,
the CheckDivergence maxima, the stop code and the final diagnostics.

The mode kθ = kz = 0 of the pressure equation is singular; the reference
solves it with LAPACK's roundoff pivot, which adds an arbitrary constant to
φ of that mode every substep (SolvePressureCorrection.F90:137-141).  Through
CorrectPressure (`amm = apph(kc)`, CorrectPressure.F90:40) that constant
reaches pr only as a function of the radial index.  The pressure is
therefore compared with the θ-z mean of every radial level removed; the
velocities do not see the constant (only differences of φ enter them).
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load():
    with open(os.path.join(GOLDEN, "reference_runs.json")) as f:
        meta = json.load(f)
    z = np.load(os.path.join(GOLDEN, "reference_runs.npz"))
    return meta["cases"], {k: z[k] for k in z.files}


CASES, DATA = load()
# runs of the main loop (the restart cases keep only their interpolated start)
CASE_NAMES = [c["name"] for c in CASES if not c.get("old_grid")]
STATS_CASES = [c["name"] for c in CASES if c.get("stats")]
RESTART_CASES = [c["name"] for c in CASES if c.get("old_grid")]
CREATED_START_CASES = [c["name"] for c in CASES if int(c["bou"]["nread"]) == 0]
FILES_CASES = [c["name"] for c in CASES if c.get("files")]
ROUTINE_CASES = [n for n in CASE_NAMES if any(k.startswith(f"{n}/routine:") for k in DATA)]
# statistics in the order of the fixture (StatRoutines.F90 names) and of
# the library's STATS list
STAT_NAMES = ["vt_me", "vr_me", "vz_me", "wt_me", "wr_me", "wz_me", "vt_rms", "vr_rms", "vz_rms", "wt_rms", "wr_rms",
              "wz_rms", "vtvr_me", "vtvz_me", "vrvz_me", "pr_me", "pr_rms", "disste"]


def case(name):
    return next(c for c in CASES if c["name"] == name)


def ref(name, key):
    return DATA[f"{name}/{key}"]


def start_time(c):
    """The time a case's run starts at: its continua files' time, or 0 with
    IRESET = 1 (ReadFlowField.F90:144)."""
    return 0.0 if int(c["bou"]["ireset"]) else float(c.get("start_time", 0.0))


def run_bou(c):
    """bou of a case as the run sees it after ReadFlowField: TMAX counts from
    the restart time (ReadFlowField.F90:149)."""
    return dict(c["bou"], tmax=float(c["bou"]["tmax"]) + start_time(c))


def write_continua(directory, c, state, time):
    """continua_q*.h5 and continua_master.h5 of `state` on c's grid at
    `time` (the files WriteFlowField writes)."""
    import tc_gb300 as tcg
    bou = c["bou"]
    nthm, nzm, nrm = int(bou["nthm"]), int(bou["nzm"]), int(bou["nrm"])
    tcg.h5_write_scalars(os.path.join(directory, "continua_master.h5"),
                         dict(nr=nrm + 1, nth=nthm + 1, nz=nzm + 1, time=time, rint=bou["rint"], rext=bou["rext"],
                              istr=bou["istr"], str=bou["str"], alx3=bou["alx3"], lamb=bou["lamb"]),
                         ints=("nr", "nth", "nz", "istr"))
    for k, a in zip(("qt", "qr", "qz"), state[:3]):
        tcg.h5_write(os.path.join(directory, f"continua_{k}.h5"), "var", np.ascontiguousarray(a[1:-1, 1:-1, :]))


def start(c):
    """The start of a case: the reference's own initial condition for
    NREAD = 0, else the seeded field its continua files held."""
    import tc_gb300.initial as ini
    if int(c["bou"]["nread"]) == 0:
        return ini.create_initial_conditions(c["bou"])
    return ini.couette_noise(c["bou"], seed=c["seed"], amp=c["amp"])


def is_output_step(ntime, time, dt, tout):
    """main.F90:184: the step of index ntime ends in an output block."""
    return ntime == 1 or math.fmod(time, tout) < dt


def march(step, cfl, torque, c, stats=None, vstats=None, div=None, t0=0.0):
    """Advance a simulation as main.F90:152-226 does, one step at a time.

    step(ntime, time, dt) -> (code, time, dt) runs the step of index ntime;
    cfl() and torque() are CalcMaxCFL and CalcTorque of the current state;
    stats(time, dt), when given, is what an output step after TSTA runs
    (main.F90:188-198: CalcStats, CalcDissipation and the dumps due at
    that time), returning the dissipation number;
    vstats() and div(), when given, are CalcVelocityStats (vmax, rms) and
    CheckDivergence, recorded at every output step (main.F90:181,185) and,
    for div, before the loop (main.F90:125).
    t0 is the time the run starts at (a restart's, ReadFlowField.F90:144).
    Returns the per-step dt, time and CFL, the torques of the output steps,
    the dissipation numbers, vmax and divergence records, the stop code and
    the index of the last step."""
    bou = c["bou"]
    ntst = int(bou["ntst"])
    t, dt = float(t0), 0.0
    rec = dict(dt=[], time=[], cfl=[], torque=[], nute=[], vmax=[], rms=[], dmax=[])
    if div is not None:
        rec["dmax"].append(div())
    code, ntime = 0, 0
    for ntime in range(0, ntst + 1):
        rec["cfl"].append(cfl())
        code, t, dt = step(ntime, t, dt)
        rec["dt"].append(dt)
        rec["time"].append(t)
        if is_output_step(ntime, t, dt, bou["tout"]):
            if vstats is not None:
                vm, rms = vstats()
                rec["vmax"].append(tuple(vm))
                rec["rms"].append((t,) + tuple(rms))
            if div is not None:
                rec["dmax"].append(div())
            rec["torque"].append((t,) + tuple(torque()))
            if stats is not None and t > bou["tsta"]:
                rec["nute"].append((t, stats(t, dt)))
        if code != 0:
            break
    rec["code"], rec["ntime"] = code, ntime
    return rec


def relmax(a, b):
    den = float(np.abs(b).max())
    return float(np.abs(a - b).max()) / (den if den > 0 else 1.0)


def pressure_fluct(p, nrm):
    """Interior pr without the θ-z mean of each radial level."""
    a = p[1:-1, 1:-1, :nrm]
    return a - a.mean(axis=(0, 1), keepdims=True)


def field_errors(c, state):
    """Relative errors of (qt, qr, qz, pr) against the reference run: the
    interior cells (qt, qz, pr: nrm radial levels; qr: nr faces), each
    divided by the reference field's maximum; pr with the radial profile
    removed and divided by max |pr| of the reference.  Cases that keep
    only some theta planes compare those planes and the whole-field sums."""
    name = c["name"]
    nrm = int(c["bou"]["nrm"])
    planes = c.get("planes")
    out = {}
    for k, a, nk in zip(("qt", "qr", "qz", "pr"), state, (nrm, nrm + 1, nrm, nrm)):
        if planes is None:
            b = ref(name, k)
            full_b = b
        else:
            b = ref(name, k + "_planes")
            a_full = a
            a = a[planes]
            full_b = None
        if k == "pr":
            scale = float(np.abs(b[1:-1, 1:-1, :nrm]).max()) if planes is None else float(np.abs(b[:, 1:-1, :nrm]).max())
            if planes is None:
                err = float(np.abs(pressure_fluct(a, nrm) - pressure_fluct(b, nrm)).max()) / scale
            else:
                # planes keep the radial profile: compare sums of the full field instead
                err = 0.0
        else:
            if planes is None:
                ai, bi = a[1:-1, 1:-1, :nk], b[1:-1, 1:-1, :nk]
            else:
                ai, bi = a[:, 1:-1, :nk], b[:, 1:-1, :nk]
            err = relmax(ai, bi)
        if planes is not None:
            sums = _field_sums(k, a_full)
            for s, v in sums.items():
                rv = float(ref(name, s))
                err = max(err, abs(v - rv) / max(abs(rv), 1e-300) if s.endswith("sumsq") else
                          abs(v - rv) / float(ref(name, k + "_sumsq")) ** 0.5 / math.sqrt(a_full[1:-1, 1:-1].size))
        out[k] = err
    return out


def _field_sums(k, v):
    import tc_gb300.initial as ini
    a = v[1:-1, 1:-1, :]
    if k == "pr":
        a = a[..., :-1]
        a = a - a.mean(axis=(0, 1), keepdims=True)
    w = ini.uniform(99, 7, a.shape[0], a.shape[1], a.shape[2])
    return {k + "_sum": float(a.sum()), k + "_sumsq": float((a * a).sum()), k + "_wsum": float((a * w).sum())}


def torque_error(ti, to, rti, rto):
    """Relative error of inner and outer torques (scalars or records), each
    against the largest reference value of its wall, but not below 1e-9 of
    the other wall's: a torque that is that far below the other one is zero
    to the precision of the sums (a fluid at rest at the outer wall while
    the inner one spins it up), and a different summation order moves it by
    roundoff of the terms, not of the result."""
    ti, to, rti, rto = (np.atleast_1d(np.asarray(x, dtype=np.float64)) for x in (ti, to, rti, rto))
    si, so = float(np.abs(rti).max()), float(np.abs(rto).max())
    di, do = max(si, 1e-9 * so), max(so, 1e-9 * si)
    return max(float(np.abs(ti - rti).max()) / (di if di > 0 else 1.0),
               float(np.abs(to - rto).max()) / (do if do > 0 else 1.0))


def scalar_errors(c, rec):
    """Relative errors of the dt sequence, the step times, the CFL numbers
    behind dt and the output-step torques against the reference run."""
    name = c["name"]
    rdt, rtime, rcfl = ref(name, "step_dt"), ref(name, "step_time"), ref(name, "step_cfl")
    rtq = ref(name, "out_torque")
    n = len(rdt)
    assert len(rec["dt"]) == n, (len(rec["dt"]), n)
    e = dict(dt=relmax(np.array(rec["dt"]), rdt), time=relmax(np.array(rec["time"]), rtime),
             cfl=relmax(np.array(rec["cfl"]), rcfl))
    tq = np.array(rec["torque"]).reshape(-1, 3)
    assert tq.shape == rtq.shape, (tq.shape, rtq.shape)
    e["torque"] = torque_error(tq[:, 1], tq[:, 2], rtq[:, 1], rtq[:, 2]) if len(tq) else 0.0
    if rec["vmax"]:
        vm, rvm = np.array(rec["vmax"]), ref(name, "out_vmax")
        assert vm.shape == rvm.shape, (vm.shape, rvm.shape)
        e["vmax"] = max(relmax(vm[:, i], rvm[:, i]) for i in range(3))
        rr, rrr = np.array(rec["rms"]), ref(name, "out_rms")
        assert rr.shape == rrr.shape, (rr.shape, rrr.shape)
        # (the values the reference wrote to rms_vel.out, before formatting)
        e["rms"] = max(relmax(rr[:, i], rrr[:, i]) for i in range(1, 4))
    if rec["dmax"]:
        # the start's divergence (O(1) for the seeded noise) relative; after
        # the projection both sides hold roundoff, compared against the
        # start's value
        dm, rdm = np.array(rec["dmax"]), ref(name, "out_dmax")
        assert dm.shape == rdm.shape, (dm.shape, rdm.shape)
        e["dmax"] = float(np.abs(dm - rdm).max()) / float(rdm[0])
    return e


def stat_errors(c, stat, samples, rec):
    """Relative errors of the accumulated statistics (stat(name) -> (nzm,
    nrm) array in the library's naming), the sample count and the
    dissipation records against the reference run.  pr_mean is compared
    with the z-mean of every radial level removed (the singular mode's
    offset depends on the radial index only); pr_rms, which squares that
    offset into the field, is not compared."""
    import tc_gb300 as tcg
    name = c["name"]
    assert samples == int(ref(name, "stat_samples")), (samples, int(ref(name, "stat_samples")))
    out = {}
    for lib_name, fname in zip(tcg.STATS, STAT_NAMES):
        if fname == "pr_rms":
            continue
        a, b = stat(lib_name), ref(name, "stat_" + fname)
        if fname == "pr_me":
            a = a - a.mean(axis=0, keepdims=True)
            b = b - b.mean(axis=0, keepdims=True)
        out[lib_name] = relmax(a, b)
    rn = ref(name, "out_nute")
    nu = np.array(rec["nute"]).reshape(-1, 2)
    assert nu.shape == rn.shape, (nu.shape, rn.shape)
    out["nute"] = relmax(nu[:, 1], rn[:, 1])
    return out


def h5_files(name, kind="h5"):
    """The HDF5 files the reference run wrote (kind "h5") or was given
    before it started (kind "h5in"): path (relative to the run's directory)
    -> {dataset: array}."""
    out = {}
    pre = f"{name}/{kind}:"
    for k, v in DATA.items():
        if k.startswith(pre):
            path, dset = k[len(pre):].rsplit(":", 1)
            out.setdefault(path, {})[dset] = v
    return out


# The routines of a substep in TimeMarcher.F90:31-54 order, with the arrays
# each one writes (the names of the reference's arrays; "hr" is dph as
# ExplicitTermsQR leaves it, "phi" dph after SolvePressureCorrection).
ROUTINES = [("explicittermsqt", ("dq",)), ("explicittermsqr", ("hr",)), ("explicittermsqz", ("qcap",)),
            ("implicitandupdateqt", ("qt", "ru1")), ("implicitandupdateqr", ("qr", "ru2")),
            ("implicitandupdateqz", ("qz", "ru3")), ("calclocaldivergence", ("div",)),
            ("solvepressurecorrection", ("phi",)), ("correctvelocity", ("qt", "qr", "qz")),
            ("correctpressure", ("pr",))]
_REF_ARRAY = {"hr": "dph", "div": "dph", "phi": "dph"}


def routine_error(name, ns, routine, arr, mine, nrm):
    """Relative error of one routine's output in substep ns against the
    reference run.  `mine` is in the library's layout: haloed
    (nthm+2, nzm+2, nr) for qt, qr, qz, pr and dph (div, phi), plain
    (nthm, nzm, nr) for dq, qcap, ru1..ru3 and hr.  Compared are the
    levels the routine defines; phi and pr without the theta-z mean of each
    radial level (the singular mode's offset), against max |reference|.
    From substep 2 on that offset has entered pr, and the radial pressure
    gradient of ImplicitAndUpdateQR (ImplicitAndUpdateQR.F90:58) carries its
    radial differences into the theta-z mean of qr and of the divergence of
    that qr (the projection then takes it out again: CorrectVelocity leaves
    the same qr); those two are compared without their theta-z mean of each
    level too."""
    ref_ = ref(name, f"routine:{ns}:{routine}:{_REF_ARRAY.get(arr, arr)}")
    if ns >= 2 and (routine, arr) in (("implicitandupdateqr", "qr"), ("calclocaldivergence", "div")):
        nk = nrm + 1 if arr == "qr" else nrm
        a, b = mine[1:-1, 1:-1, :nk], ref_[1:-1, 1:-1, :nk]
        scale = float(np.abs(b).max())
        return float(np.abs((a - a.mean(axis=(0, 1))) - (b - b.mean(axis=(0, 1)))).max()) / scale
    if arr in ("dq", "qcap", "ru1", "ru3"):
        a, b = mine[..., :nrm], ref_[..., :nrm]
    elif arr == "ru2":
        a, b = mine[..., 1:nrm], ref_[..., 1:nrm]
    elif arr == "hr":
        a, b = mine[..., 1:nrm], ref_[1:-1, 1:-1, 1:nrm]
    elif arr == "qr":
        a, b = mine[1:-1, 1:-1, :nrm + 1], ref_[1:-1, 1:-1, :nrm + 1]
    elif arr in ("phi", "pr"):
        scale = float(np.abs(ref_[1:-1, 1:-1, :nrm]).max())
        return float(np.abs(pressure_fluct(mine, nrm) - pressure_fluct(ref_, nrm)).max()) / scale
    else:
        a, b = mine[1:-1, 1:-1, :nrm], ref_[1:-1, 1:-1, :nrm]
    return relmax(a, b)

"""The CUDA path against runs of the reference's own Fortran source.

Every case of tests/golden/reference_runs.npz (tests/refruns.py) is run on
the GPU through the C ABI (tc_run one step at a time, as main.F90:152-226
runs the loop) from the same seeded start and bou.in values:

* FP64 (the drop-in): velocities and pressure (radial profile of the
  singular mode removed) within 1e-10 of the reference's, the dt sequence,
  step times, CFL numbers, output-step torques, CalcVelocityStats maxima
  and CheckDivergence maxima within 1e-10 relative,
  the same stop code at the same step;
* the mixed forms (FP32 velocity side; FP64 or float-float pressure
  tridiagonals) on every case (the kept theta planes where a case keeps
  only some): velocities within
  1e-3 of the velocity scale and torques within 1e-4 relative, each error
  printed;
* every routine of a step's three substeps through the per-component
  entry points, each against what the reference's routine left;
* the statistics case: CalcStats / CalcDissipation accumulations within
  1e-10 of the reference's, and every HDF5 file the reference run wrote
  (slab and full-field dumps, statistics, continuation files) written
  by the library with the same names, datasets and values;
* an ensemble holding every case that runs to NTST (grouped launches, FP64
  members of different shapes): each member within 1e-10 of its reference
  run.
"""
import numpy as np
import pytest

from conftest import tc

import refruns as R

pytestmark = pytest.mark.gpu

TOL = 1e-10
TOL_MIXED_Q = 1e-3
TOL_MIXED_TORQUE = 1e-4


def gpu_march(c, precision="fp64"):
    g = tc.TaylorCouette(c["bou"], precision=precision)
    t0 = 0.0
    if c.get("start_time"):
        # a restart: the library reads the continuation files, takes their
        # time and extends TMAX by it (ReadFlowField.F90:144-149)
        import shutil
        import tempfile
        d = tempfile.mkdtemp()
        try:
            R.write_continua(d, c, R.start(c), c["start_time"])
            t0 = g.read_continua(d)
        finally:
            shutil.rmtree(d)
        assert t0 == R.start_time(c) and g.bou["tmax"] == R.run_bou(c)["tmax"]
    else:
        g.set_state(*R.start(c))

    def step(ntime, t, dt):
        code, _, t, dt = g.run(1, ntime, t, dt)
        return code, t, dt

    rec = R.march(step, g.calc_max_cfl, g.calc_torque, c, vstats=g.velocity_stats,
                  div=g.check_divergence, t0=t0)
    return g, rec


@pytest.mark.parametrize("name", R.CASE_NAMES)
def test_fp64_matches_reference_run(gpu_lib, name):
    c = R.case(name)
    g, rec = gpu_march(c)
    assert rec["code"] == int(R.ref(name, "errorcode"))
    assert rec["ntime"] == int(R.ref(name, "ntime"))
    se = R.scalar_errors(c, rec)
    fe = R.field_errors(c, g.get_state())
    print(name, {k: f"{v:.1e}" for k, v in {**fe, **se}.items()})
    for k, v in {**fe, **se}.items():
        assert v <= TOL, (k, v)
    ti, to = g.calc_torque()
    rt = R.ref(name, "final_torque")
    assert R.torque_error(ti, to, rt[1], rt[2]) <= TOL
    if rec["code"] != 169:
        assert g.check_divergence() < c["bou"]["resid"]
    g.close()


@pytest.mark.parametrize("name", R.ROUTINE_CASES)
def test_fp64_routines_match_reference_run(gpu_lib, name):
    """The per-component entry points, each right after it runs, against
    what the reference's routine of the same name left in the first step
    of the reference run (TimeMarcher.F90:31-54, three substeps): within
    1e-10 (the divergence, phi and pr compared as refruns.routine_error
    says)."""
    c = R.case(name)
    bou = R.run_bou(c)
    nrm = int(bou["nrm"])
    g = tc.TaylorCouette(bou)
    g.set_state(*R.start(c))
    g.begin_step(float(bou["dtmin"]), R.start_time(c))
    calls = {"explicittermsqt": g.explicit_terms_qt, "explicittermsqr": g.explicit_terms_qr,
             "explicittermsqz": g.explicit_terms_qz, "implicitandupdateqt": g.implicit_and_update_qt,
             "implicitandupdateqr": g.implicit_and_update_qr, "implicitandupdateqz": g.implicit_and_update_qz,
             "calclocaldivergence": g.calc_local_divergence, "solvepressurecorrection": g.solve_pressure_correction,
             "correctvelocity": g.correct_velocity, "correctpressure": g.correct_pressure}
    field = {"div": "dph", "phi": "dph"}
    worst = {}
    for ns in range(1, int(bou["nsst"]) + 1):
        g.set_substep(ns)
        for routine, arrays in R.ROUTINES:
            calls[routine]()
            for arr in arrays:
                e = R.routine_error(name, ns, routine, arr, g.get_field(field.get(arr, arr)), nrm)
                worst[f"{ns}:{routine}:{arr}"] = e
                assert e <= TOL, (ns, routine, arr, e)
    print(name, "worst", max(worst.items(), key=lambda kv: kv[1]))
    g.close()


@pytest.mark.parametrize("name", R.STATS_CASES)
def test_fp64_statistics_match_reference_run(gpu_lib, name):
    """CalcStats + CalcDissipation on the GPU at the output steps after TSTA
    (main.F90:188-190): the accumulated theta averages, the sample count and
    the dissipation numbers within 1e-10 of the reference's."""
    c = R.case(name)
    g = tc.TaylorCouette(c["bou"])
    g.set_state(*R.start(c))

    def step(ntime, t, dt):
        code, _, t, dt = g.run(1, ntime, t, dt)
        return code, t, dt

    def stats(t, dt):
        g.calc_stats()
        return g.calc_dissipation()

    rec = R.march(step, g.calc_max_cfl, g.calc_torque, c, stats=stats)
    assert rec["code"] == int(R.ref(name, "errorcode"))
    err = R.stat_errors(c, g.stat, g.stat_samples, rec)
    print(name, {k: f"{v:.1e}" for k, v in err.items()})
    for k, v in err.items():
        assert v <= TOL, (k, v)
    g.close()


@pytest.mark.parametrize("name", R.FILES_CASES)
def test_output_files_match_reference_run(gpu_lib, tmp_path, name):
    """The HDF5 files of the reference run, written by the library from the
    GPU run at the same points of the loop: the radial, theta and
    streamwise-average slabs every TFRAME2D and the full fields every
    TFRAME3D of the output steps after TSTA (main.F90:188-198: DumpRCuts,
    DumpThCuts, DumpStreamwiseAvg, DumpFlowField), WriteStats and
    WriteFlowField at the stop (QuitRoutine.F90:27-30), and the grid file
    of WriteGridInfo.  The same file
    names, the same datasets in each file with the same shapes and types
    (32-bit integers, 64-bit reals), integers equal, reals within 1e-10 of each dataset's maximum (pr_mean with the
    z-mean of every radial level removed, as for the pressure; pr_rms,
    which squares the singular mode's offset in, is compared by shape).
    With STAREAD = 1 the statistics files of an earlier run are given
    first, and both add them to the run's own (StatReadReduceWrite)."""
    import math
    import os
    from test_h5 import walk
    c = R.case(name)
    bou = c["bou"]
    g = tc.TaylorCouette(bou)
    g.set_state(*R.start(c))
    d = str(tmp_path)
    sub = {k: os.path.join(d, k) for k in ("rcuts", "thcut", "stave", "fullff", "stats")}
    for v in sub.values():
        os.makedirs(v)
    # files of an earlier run that this one reads (STAREAD = 1)
    given = R.h5_files(name, "h5in")
    for path, dsets in given.items():
        ints = {k: int(v[0]) for k, v in dsets.items() if v.dtype.kind == "i"}
        if ints:
            tc.h5_write_scalars(os.path.join(d, path), ints, ints=tuple(ints))
        else:
            (k, v), = dsets.items()
            tc.h5_write(os.path.join(d, path), k, v)

    def step(ntime, t, dt):
        code, _, t, dt = g.run(1, ntime, t, dt)
        return code, t, dt

    def stats(t, dt):
        g.calc_stats()
        nute = g.calc_dissipation()
        if math.fmod(t, bou["tframe2d"]) < dt:
            if bou["nslabr"]:
                g.dump_rcuts(sub["rcuts"], t, c["rcuts"])
            if bou["dpthcut"]:
                g.dump_thcuts(sub["thcut"], t)
            if bou["dpstave"]:
                g.dump_streamwise_avg(sub["stave"], t)
        if math.fmod(t, bou["tframe3d"]) < dt and bou["dpfullf"]:
            g.dump_flow_field(sub["fullff"], t)
        return nute

    rec = R.march(step, g.calc_max_cfl, g.calc_torque, c, stats=stats)
    assert rec["code"] == int(R.ref(name, "errorcode")) == 555
    g.write_stats(sub["stats"], readstats=bool(bou["starea"]))
    g.write_continua(d, rec["time"][-1])
    tc.h5_write_grid_info(bou, d)
    g.close()
    want = R.h5_files(name)
    got = {os.path.relpath(os.path.join(r, f), d) for r, _, fs in os.walk(d) for f in fs if f.endswith(".h5")}
    assert got == set(want) | set(given), (sorted(got ^ (set(want) | set(given))))
    worst = {}
    for path, dsets in want.items():
        mine = walk(os.path.join(d, path))
        assert set(mine) == set(dsets), (path, sorted(mine), sorted(dsets))
        for k, b in dsets.items():
            a = mine[k][2]
            assert a.shape == b.shape, (path, k, a.shape, b.shape)
            assert mine[k][1] == ("<i4" if b.dtype.kind == "i" else "<f8"), (path, k, mine[k][1])
            if b.dtype.kind == "i":
                assert np.array_equal(a, b), (path, k, a, b)
                continue
            if k == "pr_rms":
                continue
            if k == "pr_mean":
                a = a - a.mean(axis=0, keepdims=True)
                b = b - b.mean(axis=0, keepdims=True)
            worst[f"{path}:{k}"] = R.relmax(a, b)
    print(name, len(want), "files;", "worst", max(worst.items(), key=lambda kv: kv[1]))
    for k, v in worst.items():
        assert v <= TOL, (k, v)


MIXED_CASES = [n for n in R.CASE_NAMES if not R.case(n).get("start_time")]


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
@pytest.mark.parametrize("name", MIXED_CASES)
def test_mixed_against_reference_run(gpu_lib, name, precision):
    """The mixed forms on the reference's own time grid: the dt sequence of
    the reference run is imposed (each form's own CFL rule would pick a
    slightly different dt), so the difference is the precision alone."""
    c = R.case(name)
    g = tc.TaylorCouette(c["bou"], precision=precision)
    g.set_state(*R.start(c))
    times = np.concatenate([[0.0], R.ref(name, "step_time")[:-1]])
    for dt, t in zip(R.ref(name, "step_dt"), times):
        g.time_marcher(float(dt), float(t))
    st = g.get_state()
    nrm = int(c["bou"]["nrm"])
    planes = c.get("planes")
    if planes is None:
        mine = {k: a[1:-1, 1:-1] for k, a in zip(("qt", "qr", "qz"), st[:3])}
        want = {k: R.ref(name, k)[1:-1, 1:-1] for k in ("qt", "qr", "qz")}
    else:      # the theta planes the case keeps
        mine = {k: a[planes, 1:-1] for k, a in zip(("qt", "qr", "qz"), st[:3])}
        want = {k: R.ref(name, k + "_planes")[:, 1:-1] for k in ("qt", "qr", "qz")}
    scale = max(float(np.abs(want["qt"][..., :nrm]).max()), 1.0)
    err = {k: float(np.abs(mine[k][..., :nk] - want[k][..., :nk]).max()) / scale
           for k, nk in zip(("qt", "qr", "qz"), (nrm, nrm + 1, nrm))}
    ti, to = g.calc_torque()
    rt = R.ref(name, "final_torque")
    terr = R.torque_error(ti, to, rt[1], rt[2])
    print(name, precision, {k: f"{v:.1e}" for k, v in err.items()}, f"torque {terr:.1e}",
          f"div {g.check_divergence():.1e}")
    assert max(err.values()) <= TOL_MIXED_Q
    assert terr <= TOL_MIXED_TORQUE
    if int(R.ref(name, "errorcode")) != 169:
        assert g.check_divergence() < c["bou"]["resid"]
    g.close()


def test_ensemble_members_match_reference_runs(gpu_lib):
    """Grouped launches over members of different shapes, radial grids and
    dt rules: every member lands on its reference run.  (An ensemble runs
    one time scheme and no patterned slip, so the AB2 and slip cases stay
    out.)"""
    names = [n for n in R.CASE_NAMES if int(R.ref(n, "errorcode")) == 555 and R.case(n).get("planes") is None
             and int(R.case(n)["bou"]["nsst"]) == 3 and int(R.case(n)["bou"]["minstrt"]) == 0
             and not R.case(n).get("start_time")]
    assert len(names) >= 5
    ens = tc.Ensemble("fp64")
    slots, left = {}, {}
    for n in names:
        c = R.case(n)
        left[n] = int(c["bou"]["ntst"]) + 1
        slots[n] = ens.add(c["bou"], R.start(c), nsteps=left[n], dt=0.0)
    # advance to the end of the shortest remaining run, check and retire it
    # (the step counts of ensemble members are the caller's to keep)
    while slots:
        k = min(left[n] for n in slots)
        ens.step(k)
        ens.sync()
        for n in list(slots):
            left[n] -= k
            if left[n]:
                continue
            c = R.case(n)
            done, t, dt, code = ens.status_full(slots[n])
            assert done == int(c["bou"]["ntst"]) + 1
            assert abs(t - float(R.ref(n, "final_time"))) <= TOL * float(R.ref(n, "final_time"))
            fe = R.field_errors(c, ens.member(slots[n]).get_state())
            print(n, {k2: f"{v:.1e}" for k2, v in fe.items()})
            for k2, v in fe.items():
                assert v <= TOL, (n, k2, v)
            ens.remove(slots.pop(n))
    ens.close()

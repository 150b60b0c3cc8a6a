"""The CPU oracle against runs of the reference's own Fortran source.

Every case of tests/golden/reference_runs.npz (see tests/refruns.py) is run
through the C++ restatement (oracle/tc_ref.cpp) one step at a time as
main.F90:152-226 runs it, from the same seeded start and bou.in values, and
compared with what the reference computed:

* velocities: 1e-12 of each field's maximum (measured: below 3e-14);
* pressure with the radial profile of the singular mode removed: 1e-11 of
  max |pr| (measured: below 2e-13);
* the dt sequence, the step times, the CFL numbers behind dt, the
  CalcTorque records and the CalcVelocityStats maxima of the output steps:
  1e-12 relative; the CheckDivergence maxima (the start's and, after the
  projection, the output steps' roundoff) within 1e-12 of the start's;
* the stop code and the index of the last step: equal;
* the final CheckDivergence below RESID in both.

This pins the oracle that the GPU parity tests use to the reference itself.
"""
import math
import os

import numpy as np
import pytest

import refruns as R

TOL_Q = 1e-12
TOL_P = 1e-11
TOL_S = 1e-12


def oracle_march(oracle, c):
    o = oracle.CppOracle(R.run_bou(c))
    o.set_state(*R.start(c))

    def step(ntime, t, dt):
        return o.run(ntime, 1, t, dt)

    rec = R.march(step, o.calc_max_cfl, o.calc_torque, c, vstats=o.velocity_stats,
                  div=o.check_divergence, t0=R.start_time(c))
    return o, rec


@pytest.mark.parametrize("name", R.CASE_NAMES)
def test_oracle_matches_reference_run(oracle, name):
    c = R.case(name)
    o, rec = oracle_march(oracle, c)
    assert rec["code"] == int(R.ref(name, "errorcode"))
    assert rec["ntime"] == int(R.ref(name, "ntime"))
    se = R.scalar_errors(c, rec)
    fe = R.field_errors(c, o.state())
    print(name, {k: f"{v:.1e}" for k, v in {**fe, **se}.items()})
    for k in ("qt", "qr", "qz"):
        assert fe[k] <= TOL_Q, (k, fe[k])
    assert fe["pr"] <= TOL_P, fe["pr"]
    for k, v in se.items():
        assert v <= TOL_S, (k, v)
    ti, to = o.calc_torque()
    rt = R.ref(name, "final_torque")
    assert R.torque_error(ti, to, rt[1], rt[2]) <= TOL_S
    resid = c["bou"]["resid"]
    if rec["code"] != 169:
        assert o.check_divergence() < resid and float(R.ref(name, "final_dmax")) < resid
    assert abs(o.calc_max_cfl() - float(R.ref(name, "final_cfl"))) <= TOL_S * float(R.ref(name, "final_cfl"))


@pytest.mark.parametrize("name", R.ROUTINE_CASES)
def test_oracle_routines_match_reference_run(oracle, name):
    """Every routine of the three substeps of the first step, each right
    after it runs, against what the same routine left in the reference run
    (TimeMarcher.F90:31-54): within 1e-12; the divergence (a difference of
    nearly equal fluxes times 1/(al dt)), phi and pr (radial profile of the
    singular mode removed) within 1e-11."""
    c = R.case(name)
    bou = R.run_bou(c)
    nrm = int(bou["nrm"])
    o = oracle.CppOracle(bou)
    o.set_state(*R.start(c))
    o.call("begin_step", float(bou["dtmin"]), R.start_time(c))
    calls = {"explicittermsqt": ["explicit_terms_qt"], "explicittermsqr": ["explicit_terms_qr"],
             "explicittermsqz": ["explicit_terms_qz"],
             "implicitandupdateqt": ["implicit_rhs_qt", "solve_imp_eqn_update_qt"],
             "implicitandupdateqr": ["implicit_rhs_qr", "solve_imp_eqn_update_qr"],
             "implicitandupdateqz": ["implicit_rhs_qz", "solve_imp_eqn_update_qz"],
             "calclocaldivergence": ["calc_local_divergence"], "solvepressurecorrection": ["solve_pressure_correction"],
             "correctvelocity": ["correct_velocity"], "correctpressure": ["correct_pressure"]}
    which = {"dq": oracle.DQ, "hr": oracle.DPH, "qcap": oracle.QCAP, "qt": oracle.QT, "qr": oracle.QR,
             "qz": oracle.QZ, "ru1": oracle.RU1, "ru2": oracle.RU2, "ru3": oracle.RU3, "div": oracle.DPH,
             "phi": oracle.DPH, "pr": oracle.PR}
    worst = {}
    for ns in range(1, int(bou["nsst"]) + 1):
        o.call("set_substep", ns)
        for routine, arrays in R.ROUTINES:
            for f in calls[routine]:
                o.call(f)
            for arr in arrays:
                mine = o.get(which[arr])
                if arr == "hr":
                    mine = mine[1:-1, 1:-1, :]
                e = R.routine_error(name, ns, routine, arr, mine, nrm)
                worst[f"{ns}:{routine}:{arr}"] = e
                assert e <= (TOL_P if arr in ("div", "phi", "pr") else TOL_Q), (ns, routine, arr, e)
            if routine == "implicitandupdateqz":
                for w in (oracle.QT, oracle.QR, oracle.QZ):
                    o.call("update_halo", w)
            elif routine == "solvepressurecorrection":
                o.call("update_halo", oracle.DPH)
            elif routine == "correctpressure":
                for w in (oracle.QT, oracle.QR, oracle.QZ, oracle.PR):
                    o.call("update_halo", w)
    print(name, "worst", max(worst.items(), key=lambda kv: kv[1]))


NP_CASES = [n for n in R.CASE_NAMES
            if R.case(n)["bou"]["minstrt"] * R.case(n)["bou"]["multmin"] == 0 and R.case(n).get("planes") is None
            and int(R.case(n)["bou"]["nthm"]) * int(R.case(n)["bou"]["nzm"]) * int(R.case(n)["bou"]["nrm"]) <= 4096
            and not R.case(n).get("start_time")]


@pytest.mark.parametrize("name", NP_CASES)
def test_numpy_oracle_matches_reference_run(name):
    """The second restatement (oracle/tc_np.py: whole-array NumPy, LAPACK
    through SciPy with the reference's roundoff pivot of the singular mode)
    on the reference's own dt sequence: velocities within 1e-12 of the
    reference run's, the pressure (radial profile removed) within 1e-10."""
    pytest.importorskip("scipy")
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(R.GOLDEN), "..", "oracle"))
    import tc_np
    c = R.case(name)
    n = tc_np.NpOracle(c["bou"], pin_mode00=False)
    n.set_state(*R.start(c))
    times = np.concatenate([[0.0], R.ref(name, "step_time")[:-1]])
    for dt, t in zip(R.ref(name, "step_dt"), times):
        n.time_marcher(float(dt), float(t))
    fe = R.field_errors(c, (n.qt, n.qr, n.qz, n.pr))
    print(name, {k: f"{v:.1e}" for k, v in fe.items()})
    for k in ("qt", "qr", "qz"):
        assert fe[k] <= TOL_Q, (k, fe[k])
    assert fe["pr"] <= 1e-10, fe["pr"]


@pytest.mark.parametrize("name", R.STATS_CASES)
def test_oracle_statistics_match_reference_run(oracle, name):
    """CalcStats + CalcDissipation at the output steps after TSTA
    (main.F90:188-190): the accumulated theta averages, the sample count and
    the dissipation numbers within 1e-12 of the reference's (pr_mean, radial
    profile removed, within the pressure tolerance)."""
    import tc_gb300 as tcg
    c = R.case(name)
    o = oracle.CppOracle(c["bou"])
    o.set_state(*R.start(c))

    def step(ntime, t, dt):
        return o.run(ntime, 1, t, dt)

    def stats(t, dt):
        o.calc_stats()
        return o.calc_dissipation()

    rec = R.march(step, o.calc_max_cfl, o.calc_torque, c, stats=stats)
    assert rec["code"] == int(R.ref(name, "errorcode"))
    err = R.stat_errors(c, lambda n: o.stat(tcg.STATS.index(n)), o.stat_samples(), rec)
    print(name, {k: f"{v:.1e}" for k, v in err.items()})
    for k, v in err.items():
        assert v <= (TOL_P if k == "pr_mean" else TOL_Q), (k, v)


@pytest.mark.parametrize("name", R.CREATED_START_CASES)
def test_created_initial_conditions_match_reference_run(name):
    """NREAD = 0: the start CreateInitialConditions built in the reference
    run (qt = 0, sinusoidal qr and qz, the inner-wall face of qr included)
    and the host restatement agree bit for bit on the interior."""
    import tc_gb300.initial as ini
    c = R.case(name)
    for k, a in zip(("qt", "qr", "qz"), ini.create_initial_conditions(c["bou"])[:3]):
        np.testing.assert_array_equal(a[1:-1, 1:-1], R.ref(name, "start_" + k)[1:-1, 1:-1], err_msg=k)


def test_grid_arrays_match_reference_runs():
    """The library's CreateGrid / InitPressureSolver arrays (host code, the
    same the device uses) equal the reference's, bit for bit, for every
    case's grid (ISTR 0, 4, 6, several STR3, NRM, NTM, NZM, RINT/REXT, LAMB,
    ALX3D); ak1 and ak3 over the entries the reference sets."""
    from conftest import tc
    for name in R.CASE_NAMES:
        bou = R.case(name)["bou"]
        for g in tc.GRID_ARRAYS:
            a, b = tc.grid_array(bou, g), R.ref(name, "grid_" + g)
            m = {"ak1": int(bou["nthm"]), "ak3": int(bou["nzm"])}.get(g, len(b))
            assert len(a) >= m, (name, g, len(a), m)
            np.testing.assert_array_equal(a[:m], b[:m], err_msg=f"{name} {g}")


def test_bou_in_of_every_case_reads_back(tmp_path):
    """The bou.in text each reference run read (ReadInputFile.F90), parsed
    by the library's reader, gives the case's values exactly."""
    from conftest import tc
    import sys
    sys.path.insert(0, R.GOLDEN)
    import make_reference_runs as M
    for c in R.CASES:
        p = tmp_path / f"{c['name']}.in"
        p.write_text(M.bou_text(c["bou"]))
        got = tc.read_bou(str(p))
        for k, v in c["bou"].items():
            assert got[k] == v, (c["name"], k, got[k], v)


def write_old_continua(directory, c):
    """The restart files of the restart case: the seeded start on the old
    grid written as continua_*.h5 (interior cells, C order)."""
    import tc_gb300 as tcg
    import tc_gb300.initial as ini
    obou = dict(c["bou"], **c["old_grid"])
    oq = ini.couette_noise(obou, seed=c["seed"], amp=c["amp"])
    nthm, nzm, nrm = obou["nthm"], obou["nzm"], obou["nrm"]
    tcg.h5_write_scalars(os.path.join(directory, "continua_master.h5"),
                         dict(nr=nrm + 1, nth=nthm + 1, nz=nzm + 1, time=0.0, rint=obou["rint"],
                              rext=obou["rext"], istr=obou["istr"], str=obou["str"], alx3=obou["alx3"],
                              lamb=obou["lamb"]), ints=("nr", "nth", "nz", "istr"))
    for k, a in zip(("qt", "qr", "qz"), oq[:3]):
        tcg.h5_write(os.path.join(directory, f"continua_{k}.h5"), "var", np.ascontiguousarray(a[1:-1, 1:-1, :]))


@pytest.mark.parametrize("name", R.RESTART_CASES)
def test_restart_interpolation_matches_reference_run(tmp_path, name):
    """ReadFlowField + interp.F90 onto a finer grid (the reference's run read
    continua files of the coarser grid): the library's loader gives the
    reference's start bit for bit at every point the reference defines.
    Where the reference's interpolation reads unset halo corners of the old
    field (its value there depends on uninitialised memory) the fixture
    holds a second run with those corners zeroed, and the loader matches
    that run bit for bit too."""
    from conftest import tc
    c = R.case(name)
    write_old_continua(str(tmp_path), c)
    q = tc.h5_load_continua(c["bou"], str(tmp_path))[:3]
    for k, a in zip(("qt", "qr", "qz"), q):
        b, m = R.ref(name, "start_" + k), R.ref(name, "start_defined_" + k)
        ai, bi, mi = a[1:-1, 1:-1], b[1:-1, 1:-1], m[1:-1, 1:-1]
        assert mi.sum() > 0.9 * mi.size
        np.testing.assert_array_equal(ai[mi], bi[mi], err_msg=k)
        np.testing.assert_array_equal(ai[~mi], bi[~mi], err_msg=k)


@pytest.mark.parametrize("name", R.FILES_CASES)
def test_grid_info_file_matches_reference_run(tmp_path, name):
    """WriteGridInfo (cordin_info.h5: rm, rc, tm, zm of CreateGrid) as the
    reference run wrote it: the same datasets, bit for bit."""
    from conftest import tc
    from test_h5 import walk
    c = R.case(name)
    tc.h5_write_grid_info(c["bou"], str(tmp_path))
    mine = walk(str(tmp_path / "cordin_info.h5"))
    want = R.h5_files(name)["cordin_info.h5"]
    assert set(mine) == set(want)
    for k, b in want.items():
        assert mine[k][1] == "<f8"
        np.testing.assert_array_equal(mine[k][2], b, err_msg=k)


def test_cases_cover_the_stop_codes_and_forms():
    """The fixtures hold runs that end with 555 (NTST reached), 333 (TMAX)
    166 (dt below DTMIN), 266 (velocities above VMAX) and 169 (divergence
    above RESID), RK3 and AB2, the three radial grids, fixed and
    variable dt, rotation, the oscillating cylinder and patterned slip."""
    codes = {int(R.ref(n, "errorcode")) for n in R.CASE_NAMES}
    assert {555, 333, 166, 266, 169} <= codes
    bous = [c["bou"] for c in R.CASES]
    assert {0, 4, 6} <= {int(b["istr"]) for b in bous}
    assert {1, 3} <= {int(b["nsst"]) for b in bous}
    assert any(b["romeg"] != 0 for b in bous) and any(b["sizepert"] != 0 for b in bous)
    assert any(b["minstrt"] * b["multmin"] != 0 for b in bous)
    assert any(b["dtmin"] < b["dtmax"] for b in bous) and any(b["dtmin"] == b["dtmax"] for b in bous)
    assert any((b["nthm"], b["nzm"], b["nrm"]) == (64, 64, 64) for b in bous)
    assert R.STATS_CASES and R.RESTART_CASES and R.FILES_CASES and R.CREATED_START_CASES


REF_DIR = os.environ.get("TC_REFERENCE_DIR", "/root/reference")


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF_DIR, "TimeMarcher.F90")),
                    reason="the reference tree is not on this machine")
@pytest.mark.parametrize("name", ["stops_at_tmax", "routine_outputs_of_one_step", "statistics_and_dumps",
                                  "restart_interpolated_from_coarser_grid"])
def test_fixture_reproduces_from_the_reference_source(name):
    """Re-run small cases through the Fortran translator and get the
    committed fixture back bit for bit (every key of the case)."""
    pytest.importorskip("scipy")
    import sys
    sys.path.insert(0, R.GOLDEN)
    import make_reference_runs as M
    c = next(x for x in M.CASES if x["name"] == name)
    out = M.run_case(REF_DIR, c)
    assert set(out) == {k.split("/", 1)[1] for k in R.DATA if k.startswith(name + "/")}
    for k, v in out.items():
        np.testing.assert_array_equal(v, R.ref(c["name"], k), err_msg=k)

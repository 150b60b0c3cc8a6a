"""Ensembles: unevenly sized runs advanced together by grouped launches.

A member's result must not depend on the company it keeps: the same run
alone and in a mix of other runs gives bit-identical fields (tolerance 0),
for every tile shape, and matches the single-run path (tc_time_marcher with
the same dt) to roundoff: 1e-12 relative in FP64; for the mixed form 1e-6 of
the velocity scale (the grouped and single-run kernels are compiled apart,
so their FP32 contractions may round differently, and the pressure solve
spreads such last-bit differences over the field).
"""
import numpy as np
import pytest

from conftest import make_bou, rel_err, tc

import tc_gb300.initial as ini

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def member(nthm, nzm, nrm, eta=0.7, ren=1000.0, **kw):
    """An instance of the ensemble workloads: RINT = 1, REXT = 1/eta."""
    return make_bou(nthm=nthm, nzm=nzm, nrm=nrm, rint=1.0, rext=1.0 / eta, ren=ren, istr=0, idtv=0,
                    limitCFL=0.8, dtmin=1e-6, dtmax=1e-2, **kw)


MIX = [member(32, 48, 32, 0.6, 800.0), member(64, 32, 48, 0.8, 3000.0), member(48, 48, 16, 0.5, 600.0),
       member(16, 64, 64, 0.9, 4000.0), member(96, 24, 32, 0.7, 1500.0)]
PROBE = member(48, 40, 32, 0.75, 2000.0)


def start(bou, seed):
    return ini.couette_noise(bou, seed=seed)


def run_members(precision, bous, seeds, nsteps, dts, tune=None):
    ens = tc.Ensemble(precision)
    if tune:
        ens.tune(*tune)
    slots = [ens.add(b, start(b, s), nsteps=nsteps, dt=dt) for b, s, dt in zip(bous, seeds, dts)]
    ens.step(nsteps)
    ens.sync()
    out = [ens.member(s).get_state() for s in slots]
    stat = [ens.status(s) for s in slots]
    ens.close()
    return out, stat


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_alone_and_in_the_mix_are_identical(gpu_lib, precision):
    dt = 2e-3
    alone, st_alone = run_members(precision, [PROBE], [7], 6, [dt])
    mixed, st_mix = run_members(precision, MIX[:2] + [PROBE] + MIX[2:], [1, 2, 7, 3, 4, 5], 6,
                                [1e-3, 3e-3, dt, 2e-3, 1e-3, 2e-3])
    for a, b in zip(alone[0], mixed[2]):
        assert np.array_equal(a, b)
    assert st_alone[0] == st_mix[2] == (6, pytest.approx(6 * dt))
    # other tile shapes: same arithmetic, same bits
    for tune in [(64, 1), (256, 4), (128, 32)]:
        again, _ = run_members(precision, MIX[:2] + [PROBE] + MIX[2:], [1, 2, 7, 3, 4, 5], 6,
                               [1e-3, 3e-3, dt, 2e-3, 1e-3, 2e-3], tune=tune)
        for a, b in zip(alone[0], again[2]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_members_match_the_single_run_path(gpu_lib, precision):
    bous = [PROBE] + MIX
    seeds = [7, 1, 2, 3, 4, 5]
    dts = [2e-3, 1e-3, 3e-3, 2e-3, 1e-3, 2e-3]
    nsteps = 5
    ens_out, _ = run_members(precision, bous, seeds, nsteps, dts)
    for b, s, dt, got in zip(bous, seeds, dts, ens_out):
        g = tc.TaylorCouette(b, precision=precision)
        g.set_state(*start(b, s))
        t = 0.0
        for _ in range(nsteps):
            g.time_marcher(dt, t)
            t += dt
        want = g.get_state()
        g.close()
        nrm = b["nrm"]
        u = float(np.abs(want[0][1:-1, 1:-1, :nrm]).max())
        for a, w, nk in zip(got[:3], want[:3], (nrm, nrm + 1, nrm)):
            if precision == "fp64":
                assert rel_err(a, w, nk=nk) < TOL_FP64
            else:
                assert rel_err(a, w, nk=nk, scale=u) < 1e-6


def test_fp64_member_matches_oracle_twenty_steps(gpu_lib, oracle):
    b = PROBE
    st = start(b, 7)
    ens = tc.Ensemble("fp64")
    s = ens.add(b, st, nsteps=20, dt=2e-3)
    ens.step(20)
    got = ens.member(s).get_state()
    ens.close()
    o = oracle.CppOracle(b)
    o.set_state(*st)
    t = 0.0
    for _ in range(20):
        o.time_marcher(2e-3, t)
        t += 2e-3
    want = o.state()
    nrm = b["nrm"]
    for a, w, nk in zip(got[:3], want[:3], (nrm, nrm + 1, nrm)):
        assert rel_err(a, w, nk=nk) < 1e-10


def test_admission_retirement_and_slot_reuse(gpu_lib):
    ens = tc.Ensemble("fp64")
    a = ens.add(MIX[0], start(MIX[0], 1), dt=1e-3)
    b = ens.add(PROBE, start(PROBE, 7), dt=2e-3)
    ens.step(2)
    assert ens.count == 2 and ens.cells == sum(x["nthm"] * x["nzm"] * x["nrm"] for x in (MIX[0], PROBE))
    ens.remove(a)
    assert ens.count == 1
    c = ens.add(MIX[1], start(MIX[1], 2), dt=3e-3)
    assert c == a                                   # the freed slot is reused
    ens.step(3)
    assert ens.status(b) == (5, pytest.approx(10e-3))
    assert ens.status(c) == (3, pytest.approx(9e-3))
    assert ens.launches_per_step == 2 + 8 * 3 + 1
    # the probe went through 5 steps, 2 of them beside another member
    got = ens.member(b).get_state()
    ens.close()
    alone, _ = run_members("fp64", [PROBE], [7], 5, [2e-3])
    for x, y in zip(got, alone[0]):
        assert np.array_equal(x, y)


def test_cfl_dt_rule_and_rejections(gpu_lib):
    b = member(32, 32, 32, 0.7, 1000.0)
    st = start(b, 9)
    g = tc.TaylorCouette(b)
    g.set_state(*st)
    cfl = g.calc_max_cfl()
    g.close()
    ens = tc.Ensemble("fp64")
    s = ens.add(b, st, dt=0.0)
    ens.step(1)
    n, t = ens.status(s)
    assert n == 1 and t == pytest.approx(min(b["limitCFL"] / cfl, b["dtmax"]), rel=1e-12)
    with pytest.raises(tc.TCError):
        ens.add(dict(b, minstrt=2, minstrz=2, multmin=1), st)
    with pytest.raises(tc.TCError):
        ens.add(dict(b, nsst=1), st)
    with pytest.raises(tc.TCError):
        ens.tune(100, 0)
    ens.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_variable_dt_member_follows_the_reference_loop(gpu_lib, precision):
    """dt <= 0 with IDTV = 1: CalcMaxCFL and the main.F90 dt rule every step,
    as tc_run does for a single run."""
    b = dict(PROBE, idtv=1, limitCFL=0.8, dtmin=1e-4, dtmax=5e-3, resid=1e3)
    st = start(b, 7)
    ens = tc.Ensemble(precision)
    s_fix = ens.add(MIX[0], start(MIX[0], 1), dt=1e-3)
    s_var = ens.add(b, st, dt=0.0)
    ens.step(8)
    n, t, dt, code = ens.status_full(s_var)
    got = ens.member(s_var).get_state()
    assert ens.status(s_fix) == (8, pytest.approx(8e-3))
    ens.close()
    g = tc.TaylorCouette(b, precision=precision)
    g.set_state(*st)
    code_g, n_g, t_g, dt_g = g.run(8, 0, 0.0)
    want = g.get_state()
    g.close()
    assert code == code_g == 0 and n == n_g == 8
    assert t == pytest.approx(t_g, rel=1e-12) and dt == pytest.approx(dt_g, rel=1e-12)
    assert dt > b["dtmin"]                           # the CFL rule took over after the first steps
    nrm = b["nrm"]
    u = float(np.abs(want[0][1:-1, 1:-1, :nrm]).max())
    for a, w, nk in zip(got[:3], want[:3], (nrm, nrm + 1, nrm)):
        if precision == "fp64":
            assert rel_err(a, w, nk=nk) < TOL_FP64
        else:
            assert rel_err(a, w, nk=nk, scale=u) < 1e-6

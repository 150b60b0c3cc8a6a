"""The persistent ensemble schedule: one cooperative launch per RK substep.

It runs the same device bodies over the same work lists as the grouped
schedule, but the two schedules' kernels are compiled apart, so the
compiler may contract multiply-adds differently in each: every member's
fields agree with the grouped schedule's to 1e-12 relative in FP64 and 1e-6
of the velocity scale in the mixed form (as between the grouped and
single-run kernels), with fixed and variable dt and across admissions and
retirements.  Within the persistent schedule a member alone and in a mix is
bit-identical in both precisions.  Its grid-barrier waits are bounded: a
barrier that cannot complete makes every wait run out, the next sync reports
3001, the failed step leaves the fields as they were and later steps run
normally.
"""
import time

import numpy as np
import pytest

from conftest import rel_err, tc
from test_gpu_ensemble import MIX, PROBE, start

pytestmark = pytest.mark.gpu

VAR = dict(PROBE, nthm=32, nzm=32, nrm=24, idtv=1, limitCFL=0.8, dtmin=1e-4, dtmax=5e-3, resid=1e3)


def run(precision, schedule, bous, seeds, dts, nsteps, rows=0, blocks_per_sm=0):
    ens = tc.Ensemble(precision)
    ens.tune(128, rows, schedule, blocks_per_sm)
    slots = [ens.add(b, start(b, s), nsteps=nsteps, dt=dt) for b, s, dt in zip(bous, seeds, dts)]
    ens.step(nsteps)
    ens.sync()
    out = [ens.member(s).get_state() for s in slots]
    stat = [ens.status_full(s) for s in slots]
    info = (ens.launches_per_step, ens.persistent_blocks, ens.schedule)
    ens.close()
    return out, stat, info


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_persistent_matches_grouped(gpu_lib, precision):
    bous = MIX[:2] + [PROBE, VAR] + MIX[2:]
    seeds = [1, 2, 7, 11, 3, 4, 5]
    dts = [1e-3, 3e-3, 2e-3, 0.0, 2e-3, 1e-3, 2e-3]      # 0.0 with IDTV = 1: variable dt
    g_out, g_st, g_info = run(precision, "grouped", bous, seeds, dts, 6)
    p_out, p_st, p_info = run(precision, "persistent", bous, seeds, dts, 6)
    assert g_info[0] == 2 + 8 * 3 + 2 and g_info[2] == "grouped"
    assert p_info[0] == 3 and p_info[1] > 0 and p_info[2] == "persistent"
    if precision == "fp64":
        assert [s[0] for s in p_st] == [s[0] for s in g_st] and [s[3] for s in p_st] == [s[3] for s in g_st]
        for (_, t1, d1, _), (_, t2, d2, _) in zip(g_st, p_st):
            assert t1 == pytest.approx(t2, rel=1e-12) and d1 == pytest.approx(d2, rel=1e-12)
        for b, a, w in zip(bous, p_out, g_out):
            nrm = b["nrm"]
            for x, y, nk in zip(a[:3], w[:3], (nrm, nrm + 1, nrm)):
                assert rel_err(x, y, nk=nk) < 1e-12
        return
    for (n1, t1, d1, c1), (n2, t2, d2, c2) in zip(g_st, p_st):
        assert (n1, c1) == (n2, c2) and t1 == pytest.approx(t2, rel=1e-6) and d1 == pytest.approx(d2, rel=1e-6)
    for b, a, w in zip(bous, p_out, g_out):
        nrm = b["nrm"]
        u = float(np.abs(w[0][1:-1, 1:-1, :nrm]).max())
        for x, y, nk in zip(a[:3], w[:3], (nrm, nrm + 1, nrm)):
            assert rel_err(x, y, nk=nk, scale=u) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_persistent_alone_and_in_the_mix_are_identical(gpu_lib, precision):
    alone, st_a, _ = run(precision, "persistent", [PROBE], [7], [2e-3], 5)
    for rows, bps in ((0, 0), (2, 1), (8, 2)):
        mix, st_m, info = run(precision, "persistent", MIX[:3] + [PROBE], [1, 2, 3, 7], [1e-3, 3e-3, 2e-3, 2e-3], 5,
                              rows=rows, blocks_per_sm=bps)
        if bps:
            assert info[1] % bps == 0 and info[1] // bps >= 100      # blocks = SMs x cap
        assert st_a[0] == st_m[3]
        for x, y in zip(alone[0], mix[3]):
            assert np.array_equal(x, y)


def test_persistent_admission_and_retirement(gpu_lib):
    def scenario(schedule):
        ens = tc.Ensemble("fp64")
        ens.set_schedule(schedule)
        a = ens.add(MIX[0], start(MIX[0], 1), dt=1e-3)
        b = ens.add(PROBE, start(PROBE, 7), dt=2e-3)
        ens.step(2)
        ens.remove(a)
        c = ens.add(MIX[3], start(MIX[3], 4), dt=2e-3)
        ens.step(3)
        ens.sync()
        out = [ens.member(s).get_state() for s in (b, c)]
        st = [ens.status(s) for s in (b, c)]
        ens.close()
        return out, st

    g, gs = scenario("grouped")
    p, ps = scenario("persistent")
    assert ps[0] == (5, pytest.approx(10e-3)) and ps[1] == (3, pytest.approx(6e-3))
    for b, a, w in zip((PROBE, MIX[3]), p, g):
        nrm = b["nrm"]
        for x, y, nk in zip(a[:3], w[:3], (nrm, nrm + 1, nrm)):
            assert rel_err(x, y, nk=nk) < 1e-12


def test_barrier_timeout_is_reported_and_recovered(gpu_lib):
    bous = [MIX[0], PROBE]
    ens = tc.Ensemble("fp64")
    ens.set_schedule("persistent")
    slots = [ens.add(b, start(b, s), dt=dt) for b, s, dt in zip(bous, [1, 7], [1e-3, 2e-3])]
    ens.step(1)
    ens.sync()
    before = [ens.member(s).get_state() for s in slots]
    ens.set_barrier_timeout(0.2)
    ens.stall_next_barrier()
    t0 = time.perf_counter()
    ens.step(2)
    with pytest.raises(tc.TCError) as ei:
        ens.sync()
    waited = time.perf_counter() - t0
    assert ei.value.code == 3001
    assert waited < 30.0
    # the failed steps stopped at their first barrier: fields and step counts unchanged
    for s, want in zip(slots, before):
        got = ens.member(s).get_state()
        for x, y in zip(got, want):
            assert np.array_equal(x, y)
    assert [ens.status(s)[0] for s in slots] == [1, 1]
    # the barrier was reset: the next steps run as an uninterrupted run's would
    ens.step(1)
    ens.sync()
    after = [ens.member(s).get_state() for s in slots]
    ens.close()
    ref, st, _ = run("fp64", "persistent", bous, [1, 7], [1e-3, 2e-3], 2)
    assert [x[0] for x in st] == [2, 2]
    for a, b in zip(after, ref):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_schedule_rejections(gpu_lib):
    ens = tc.Ensemble("fp64")
    with pytest.raises(ValueError):
        ens.set_schedule("fused")
    with pytest.raises(tc.TCError):
        ens.stall_next_barrier()                   # grouped schedule: no barrier
    with pytest.raises(tc.TCError):
        ens.set_barrier_timeout(0.0)
    ens.close()

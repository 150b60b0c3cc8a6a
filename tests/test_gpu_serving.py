"""Serving on the GPU: runs that arrive while others are on the device join
the ensemble, and each result is the same as the run alone (bit-identical
fields; the mixed form's torque within 1e-4 of the FP64 run)."""
import numpy as np
import pytest

from conftest import tc

import tc_gb300.initial as ini
import tc_gb300.serving as sv

pytestmark = pytest.mark.gpu


def small_requests():
    shapes = [(32, 48, 32), (48, 32, 16), (16, 64, 24), (64, 16, 32), (32, 32, 48), (48, 48, 16)]
    steps = [40, 23, 57, 31, 45, 19]
    reqs = []
    for i, ((a, b, c), n) in enumerate(zip(shapes, steps)):
        bou = sv.ensemble_member_bou(a, b, c, 0.5 + 0.07 * i, 600.0 + 500.0 * i, idtv=1)
        bou["dtmin"], bou["dtmax"] = 1e-4, 5e-3
        reqs.append(sv.Request(i, 0.0, bou, 50 + i, n))
    return reqs


def state_of(r):
    return ini.couette_noise(r.bou, seed=r.seed)


def alone(precision, r):
    ens = tc.Ensemble(precision)
    s = ens.add(r.bou, state_of(r), nsteps=r.nsteps, dt=0.0)
    ens.step(r.nsteps)
    m = ens.member(s)
    out = m.get_state(), m.calc_torque()
    ens.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_served_results_equal_runs_alone(gpu_lib, precision):
    reqs = small_requests()
    # the first three arrive together; the rest arrive while those run
    srv = sv.Server(precision, hbm_budget=150e9, chunk=7, keep_states=True)
    t = {"now": 0.0}

    def clock():
        return t["now"]

    def sleep(dt):
        t["now"] += dt

    for i, r in enumerate(reqs):
        r.arrival = 0.0 if i < 3 else 1e-3 * i

    # virtual time: each chunk advances the clock, so later arrivals join
    # while the first runs are still on the device
    orig_step = tc.Ensemble.step

    def step(self, n=1):
        t["now"] += 1e-3
        return orig_step(self, n)

    tc.Ensemble.step = step
    try:
        res, stats = srv.run(reqs, state_of, clock=clock, sleep=sleep)
    finally:
        tc.Ensemble.step = orig_step
    assert stats["peak_active"] >= 4                     # runs overlapped on the device
    assert sorted(r.rid for r in res) == list(range(len(reqs)))
    for r in res:
        assert r.errorcode == 0
        want_state, want_torque = alone(precision, reqs[r.rid])
        for a, b in zip(srv.states[r.rid], want_state):
            assert np.array_equal(a, b)
        assert r.torque == want_torque
        if precision == "mixed":
            _, t64 = alone("fp64", reqs[r.rid])
            for x, y in zip(r.torque, t64):
                assert abs(x - y) <= 1e-4 * abs(y)

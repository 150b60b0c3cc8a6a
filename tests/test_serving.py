"""Serving loop scheduling on the host, against a fake ensemble and a
virtual clock (no GPU): FIFO admission against the HBM budget, continuous
batching (runs join while others are on the device), chunks cut so every
run gets exactly its requested steps, and the request generators."""
import math

import pytest

from conftest import tc

import tc_gb300.serving as sv


class FakeMember:
    def __init__(self, ens, slot):
        self.ens, self.slot = ens, slot

    def calc_torque(self):
        return (float(self.ens.steps[self.slot]), -1.0)

    def get_state(self):
        return (self.ens.steps[self.slot],)


class FakeEnsemble:
    """Records what the server asks of it; a step of k costs k * cells ns of
    virtual time."""

    def __init__(self, clock):
        self.clock = clock
        self.slots, self.steps, self.bous = {}, {}, {}
        self.log = []
        self.next = 0
        self.free = []

    def __call__(self, precision):
        return self

    def set_stream(self, s):
        pass

    def tune(self, *a):
        pass

    def add(self, bou, state, nsteps=0, dt=0.0):
        s = self.free.pop() if self.free else self._new()
        self.slots[s] = nsteps
        self.steps[s] = 0
        self.bous[s] = bou
        self.log.append(("add", s, self.clock.t, len(self.slots)))
        return s

    def _new(self):
        self.next += 1
        return self.next - 1

    def remove(self, s):
        self.log.append(("remove", s, self.clock.t, self.steps[s]))
        del self.slots[s]
        self.free.append(s)

    def step(self, k):
        cells = sum(b["nthm"] * b["nzm"] * b["nrm"] for s, b in self.bous.items() if s in self.slots)
        for s in self.slots:
            self.steps[s] += k
        self.clock.t += k * cells * 1e-9
        self.log.append(("step", k, len(self.slots)))

    def sync(self):
        pass

    def status_full(self, s):
        return self.steps[s], 0.0, 0.0, 0

    def member(self, s):
        return FakeMember(self, s)

    def close(self):
        pass


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


def serve(reqs, budget, chunk=25):
    clock = Clock()
    ens = FakeEnsemble(clock)
    srv = sv.Server("mixed", hbm_budget=budget, chunk=chunk, ensemble_factory=ens)
    res, stats = srv.run(reqs, lambda r: None, clock=clock, sleep=clock.sleep)
    return res, stats, ens


def test_every_run_gets_exactly_its_steps_and_runs_overlap():
    reqs = sv.draw_requests(12, rate=4.0, seed=3)
    res, stats, ens = serve(reqs, 150e9)
    assert sorted(r.rid for r in res) == list(range(12))
    done_steps = {e[1]: e[3] for e in ens.log if e[0] == "remove"}
    by_rid = {r.rid: r for r in res}
    for r in reqs:
        assert by_rid[r.rid].nsteps == r.nsteps
        assert by_rid[r.rid].latency > 0 and by_rid[r.rid].admitted >= r.arrival
    # every removal happened after exactly the requested steps
    removes = [e for e in ens.log if e[0] == "remove"]
    assert len(removes) == 12
    assert sorted(e[3] for e in removes) == sorted(r.nsteps for r in reqs)
    # continuous batching: some step ran with several runs on the device, and
    # some run was admitted while others were active
    assert max(e[2] for e in ens.log if e[0] == "step") > 1
    assert any(e[3] > 1 for e in ens.log if e[0] == "add")
    assert stats["cell_steps"] == sum(r.bou["nthm"] * r.bou["nzm"] * r.bou["nrm"] * r.nsteps for r in reqs)
    assert done_steps  # slots were reused or retired


def test_budget_limits_resident_runs_and_admission_is_fifo():
    reqs = sv.draw_requests(10, rate=50.0, seed=5)
    one = max(sv.estimate_bytes(r.bou, "mixed") for r in reqs)
    budget = 2.5 * one
    res, stats, ens = serve(reqs, budget)
    assert stats["peak_bytes"] <= budget
    adds = [e for e in ens.log if e[0] == "add"]
    assert len(adds) == 10
    adm = [r.admitted for r in sorted(res, key=lambda r: r.rid)]
    assert adm == sorted(adm)                                        # first come, first served
    assert any(r.admitted > r.arrival + 1e-9 for r in res)           # some run waited for memory


def test_idle_server_waits_for_arrivals():
    reqs = sv.draw_requests(3, rate=0.1, seed=11)
    res, stats, ens = serve(reqs, 150e9)
    for r in res:
        assert r.admitted >= r.arrival
    assert stats["peak_active"] >= 1


def test_request_generator_ranges():
    reqs = sv.draw_requests(200, rate=5.0, seed=1)
    for r in reqs:
        b = r.bou
        assert 64 <= b["nthm"] <= 256 and 64 <= b["nzm"] <= 256 and 64 <= b["nrm"] <= 128
        assert b["nthm"] % 2 == 0 and 100 <= r.nsteps <= 2000
        eta = b["rint"] / b["rext"]
        assert 0.5 <= eta <= 0.9 and 500 <= b["ren"] <= 1e4
        assert b["idtv"] == 1
    gaps = [b.arrival - a.arrival for a, b in zip(reqs, reqs[1:])]
    assert abs(sum(gaps) / len(gaps) - 0.2) < 0.05          # Poisson, mean 1/rate
    ens = sv.draw_ensemble(96)
    assert len(ens) == 96
    assert {b["nthm"] for b in ens} <= set(sv.FFT_SIZES)
    assert len({(b["nthm"], b["nzm"], b["nrm"]) for b in ens}) > 20      # uneven
    for b in ens:
        assert 0.5 <= b["rint"] / b["rext"] <= 0.9 and 500 <= b["ren"] <= 5000


def test_percentile():
    assert sv.percentile([1, 2, 3, 4, 5], 0.5) == 3
    assert math.isclose(sv.percentile(list(range(101)), 0.99), 99.0)

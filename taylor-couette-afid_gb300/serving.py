"""Serving loop: runs arrive over time, are admitted against an HBM budget,
stay resident on the device and advance together in one ensemble
(continuous batching: a run that arrives while others are on the GPU joins
the ensemble at the next chunk boundary, a finished run leaves it and frees
its memory for the next admission).

Also the seeded instance and request generators of the ensemble and serving
workloads.  Everything here is host-side scheduling over the C ABI
(tc_ensemble_*); the arithmetic of each run is the single-run path's.
"""
from __future__ import annotations

import dataclasses
import math
import time

import numpy as np

FFT_SIZES = (32, 48, 64, 96, 128)


def ensemble_member_bou(nthm: int, nzm: int, nrm: int, eta: float, ren: float, limit_cfl: float = 0.8,
                        idtv: int = 0, nsst: int = 3) -> dict:
    """bou.in values of one instance: inner cylinder rotating (VIROTINT = 1),
    outer at rest, RINT = 1 and REXT = 1/eta, ALX3 = 2 pi, uniform radial grid."""
    return dict(nthm=nthm, nzm=nzm, nrm=nrm, nsst=nsst, idtv=idtv, nread=1, ntst=10 ** 8, tout=1.0e9,
                tmax=1.0e9, ireset=0, walltimemax=1e9, alx3=2 * math.pi, rint=1.0, rext=1.0 / eta, istr=0,
                str=4.0, lamb=1.0, virotint=1.0, virotext=0.0, sizepert=0.0, omegapert=0.0, ren=ren, romeg=0.0,
                resid=1e3, limitCFL=limit_cfl, tsta=0.0, starea=0, dtmin=1e-6, dtmax=1.0, limitVel=1e3,
                cfllim=1.0, nslabr=0, dpthcut=0, dpstave=0, tframe2d=1.0, dpfullf=0, tframe3d=1.0,
                minstrt=0, minstrz=0, multmin=0)


def draw_ensemble(n: int, seed: int = 2024):
    """The 96-instance ensemble workload: grids drawn from {32,48,64,96,128}^3,
    radius ratio uniform in [0.5, 0.9], 1/NU log-uniform in [500, 5000],
    RK3 with CFL <= 0.8 held by the reference's dt rule every step (IDTV = 1,
    CFLMAX = 0.8).  A dt fixed once from the start's CFL number does not
    keep CFL <= 0.8: the CFL number grows 5-9x in 300 steps as the Taylor
    vortices develop, and the reference scheme then diverges (also on the
    CPU oracle), so the dt is set from the CFL of each step."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nthm, nzm, nrm = (int(rng.choice(FFT_SIZES)) for _ in range(3))
        eta = float(rng.uniform(0.5, 0.9))
        ren = float(math.exp(rng.uniform(math.log(500.0), math.log(5000.0))))
        out.append(ensemble_member_bou(nthm, nzm, nrm, eta, ren, idtv=1))
    return out


def _grid_size(rng, lo: int, hi: int) -> int:
    """A size in [lo, hi] whose FFT factors into 2, 3 and 5 (even, half too)."""
    ok = [n for n in range(lo, hi + 1, 2) if _smooth(n // 2) and _smooth(n)]
    return int(rng.choice(ok))


def _smooth(n: int) -> bool:
    for p in (2, 3, 5):
        while n % p == 0 and n > 1:
            n //= p
    return n == 1


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the experiment
    bou: dict
    seed: int
    nsteps: int


def draw_requests(n: int, rate: float, seed: int = 7):
    """The serving workload: Poisson arrivals at `rate` runs/s; grid uniform
    over 64^3 .. 256x256x128 (theta x z x r, FFT-friendly sizes), radius
    ratio in [0.5, 0.9], 1/NU log-uniform in [500, 1e4], 100..2000 RK3 steps
    with the reference's variable dt (CFLMAX = 0.8)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        nthm = _grid_size(rng, 64, 256)
        nzm = _grid_size(rng, 64, 256)
        nrm = _grid_size(rng, 64, 128)
        eta = float(rng.uniform(0.5, 0.9))
        ren = float(math.exp(rng.uniform(math.log(500.0), math.log(1.0e4))))
        steps = int(rng.integers(100, 2001))
        bou = ensemble_member_bou(nthm, nzm, nrm, eta, ren, idtv=1)
        bou["dtmin"] = 1e-4
        bou["dtmax"] = 2e-2
        out.append(Request(i, t, bou, 1000 + i, steps))
        t += float(rng.exponential(1.0 / rate))
    return out


def with_rate(reqs, rate: float, seed: int = 7):
    """The same runs with arrival times of another Poisson rate."""
    rng = np.random.default_rng(seed + 1)
    t = 0.0
    out = []
    for r in reqs:
        out.append(dataclasses.replace(r, arrival=t))
        t += float(rng.exponential(1.0 / rate))
    return out


def estimate_bytes(bou: dict, precision: str) -> int:
    """Device bytes a run holds (fields, spectra, factors), from the sizes
    tc_create_ex allocates; used for admission before the run exists."""
    nt, nz, nr = int(bou["nthm"]), int(bou["nzm"]), int(bou["nrm"])
    cells = nt * nz * nr
    faces = nt * nz * (nr + 1)
    spec = nz * (nt // 2 + 1) * nr            # complex values of the half spectrum
    modes = (nz // 2 + 1) * (nt // 2 + 1) * nr
    if precision == "fp64":
        b = 8 * (8 * cells + 3 * faces) + 16 * spec
    else:
        # FP32 q, phi, ru, rhs and the pressure copy; FP64 pressure; FP32
        # spectrum and its FP64 tridiagonal workspace
        b = 4 * (8 * cells + 3 * faces) + 8 * cells + 8 * spec + 16 * spec
    b += 2 * 8 * modes                        # pressure LU factors (FP64)
    return int(b * 1.02) + (1 << 20)


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    done: float
    nsteps: int
    cells: int
    torque: tuple
    errorcode: int

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class Server:
    """Continuous-batching server over one ensemble.

    Loop: admit every arrived run that fits the HBM budget (first come, first
    served), advance the ensemble by `chunk` steps (graph replays; runs whose
    remaining steps are fewer get them exactly, because the chunk is cut to
    the smallest remainder), retire the runs that are done (their torque is
    read from the device, their memory freed), repeat."""

    def __init__(self, precision: str = "mixed", hbm_budget: float = 150e9, chunk: int = 25,
                 tune: tuple | None = None, stream: int | None = None, ensemble_factory=None,
                 keep_states: bool = False):
        self.precision = precision
        self.budget = float(hbm_budget)
        self.chunk = int(chunk)
        self.tune = tune
        self.stream = stream
        self.keep_states = keep_states
        if ensemble_factory is None:
            import tc_gb300 as tc
            ensemble_factory = tc.Ensemble
        self.factory = ensemble_factory

    def run(self, requests, make_state, clock=time.perf_counter, sleep=time.sleep, log=None):
        """Serve `requests` (arrival times relative to the call); make_state(r)
        gives a run's start.  Returns (results, stats)."""
        ens = self.factory(self.precision)
        if self.stream is not None:
            ens.set_stream(self.stream)
        if self.tune:
            ens.tune(*self.tune)
        self.states = {}
        pending = sorted(requests, key=lambda r: r.arrival)
        active = {}          # slot -> [request, admitted, steps_left, bytes]
        used = 0
        results = []
        cell_steps = 0
        t0 = clock()
        peak_active, peak_bytes = 0, 0
        try:
            while pending or active:
                now = clock() - t0
                # admission (FIFO, against the budget)
                while pending and pending[0].arrival <= now:
                    r = pending[0]
                    need = estimate_bytes(r.bou, self.precision)
                    if used + need > self.budget and active:
                        break
                    pending.pop(0)
                    slot = ens.add(r.bou, make_state(r), nsteps=r.nsteps, dt=0.0)
                    active[slot] = [r, clock() - t0, r.nsteps, need]
                    used += need
                peak_active = max(peak_active, len(active))
                peak_bytes = max(peak_bytes, used)
                if not active:
                    if pending:
                        wait = pending[0].arrival - (clock() - t0)
                        if wait > 0:
                            sleep(min(wait, 0.05))
                    continue
                k = min(self.chunk, min(a[2] for a in active.values()))
                ens.step(k)
                ens.sync()
                cells = sum(int(a[0].bou["nthm"]) * int(a[0].bou["nzm"]) * int(a[0].bou["nrm"])
                            for a in active.values())
                cell_steps += cells * k
                finished = []
                for slot, a in active.items():
                    a[2] -= k
                    if a[2] <= 0:
                        finished.append(slot)
                for slot in finished:
                    r, adm, _, need = active.pop(slot)
                    n, _, _, code = ens.status_full(slot)
                    m = ens.member(slot)
                    torque = m.calc_torque()
                    if self.keep_states:
                        self.states[r.rid] = m.get_state()
                    ens.remove(slot)
                    used -= need
                    done = clock() - t0
                    results.append(Result(r.rid, r.arrival, adm, done, r.nsteps,
                                          int(r.bou["nthm"]) * int(r.bou["nzm"]) * int(r.bou["nrm"]),
                                          tuple(torque), code))
                    if log:
                        log(f"run {r.rid} done at {done:.2f}s (arrived {r.arrival:.2f}s, {n} steps)")
            wall = clock() - t0
        finally:
            ens.close()
        return results, {"wall_s": wall, "cell_steps": cell_steps, "peak_active": peak_active,
                         "peak_bytes": peak_bytes}


def percentile(xs, q: float) -> float:
    xs = sorted(xs)
    if not xs:
        return float("nan")
    pos = (len(xs) - 1) * q
    lo, hi = int(math.floor(pos)), int(math.ceil(pos))
    return xs[lo] + (xs[hi] - xs[lo]) * (pos - lo)

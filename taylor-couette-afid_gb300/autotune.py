"""Schedule and tile-shape autotuner for ensembles.

The schedule of a step (grouped launches per phase, or one persistent
cooperative launch per RK substep) and the launch shape of the grouped
kernels -- threads per cell / column / mode tile and rows per theta-FFT
block -- change no arithmetic (each cell, column, mode and FFT line is
computed by the same device code whatever the schedule and tile), so they
can be chosen by timing alone.  ``tune`` builds a scratch ensemble with the
same members, times a few graph replays of every candidate and returns the
fastest; the scratch ensemble is then freed, so the runs being served never
advance during tuning.  The persistent schedule has fixed 128-thread tiles;
its candidates differ in the rows per theta-FFT item (at most 8) and in the
blocks per SM of the launch (fewer blocks: cheaper grid barriers, fewer
warps per phase).

Choices are cached per device and ensemble signature in a JSON file
(``TC_TUNE_CACHE`` or ``_build/tune_cache.json`` beside this file).
"""
from __future__ import annotations

import hashlib
import json
import os
import time

THREADS = (64, 128, 256)
ROWS = (0, 2, 4, 8, 16)
PERSISTENT_ROWS = (0, 2)
PERSISTENT_BLOCKS = (0, 2, 1)     # blocks per SM; 0 = occupancy limit
HERE = os.path.dirname(os.path.abspath(__file__))


def cache_path() -> str:
    return os.environ.get("TC_TUNE_CACHE", os.path.join(HERE, "_build", "tune_cache.json"))


def signature(precision: str, bous) -> str:
    """Members' shapes, sorted (the tile choice depends on nothing else)."""
    shapes = sorted((int(b["nthm"]), int(b["nzm"]), int(b["nrm"]), int(b["nsst"])) for b in bous)
    h = hashlib.sha1(json.dumps([precision, shapes]).encode()).hexdigest()[:16]
    return f"{precision}:{len(shapes)}:{h}"


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _device_key() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "cuda"


def candidates_all():
    """Every (threads, rows, schedule, blocks per SM) the tuner tries."""
    c = [(t, r, "grouped", 0) for t in THREADS for r in ROWS]
    c += [(128, r, "persistent", b) for r in PERSISTENT_ROWS for b in PERSISTENT_BLOCKS]
    return c


def time_shape(ens, threads: int, rows: int, steps: int, schedule: str = "grouped", blocks_per_sm: int = 0) -> float:
    """Seconds per step of `ens` with this schedule and tile shape (one
    warm-up replay, which also builds and captures the graph)."""
    ens.tune(threads, rows, schedule, blocks_per_sm)
    ens.step(1)
    ens.sync()
    t0 = time.perf_counter()
    ens.step(steps)
    ens.sync()
    return (time.perf_counter() - t0) / steps


def _label(t: int, r: int, sched: str, b: int) -> str:
    return f"{sched}:{t}x{r}" + (f"/{b}" if sched == "persistent" else "")


def _parse(label: str):
    sched, shape = label.split(":")
    shape, _, b = shape.partition("/")
    t, r = (int(x) for x in shape.split("x"))
    return t, r, sched, int(b or 0)


def tune(precision: str, bous, states, steps: int = 3, use_cache: bool = True, candidates=None):
    """Best (threads, rows, schedule, blocks per SM) for an ensemble of these
    members, and the table of measured seconds per step."""
    import tc_gb300 as tc
    key = _device_key() + "|" + signature(precision, bous)
    cache = _load() if use_cache else {}
    if use_cache and key in cache and "blocks_per_sm" in cache[key]:
        c = cache[key]
        return (c["threads"], c["rows"], c["schedule"], c["blocks_per_sm"]), c.get("table", {})
    cands = candidates or candidates_all()
    ens = tc.Ensemble(precision)
    try:
        for b, s in zip(bous, states):
            ens.add(b, s, dt=1e-6)
        table = {}
        for cand in cands:
            t, r = cand[0], cand[1]
            sched = cand[2] if len(cand) > 2 else "grouped"
            b = cand[3] if len(cand) > 3 else 0
            try:
                table[_label(t, r, sched, b)] = time_shape(ens, t, r, steps, sched, b)
            except tc.TCError:
                continue                    # not possible for these members
    finally:
        ens.close()
    if not table:
        raise RuntimeError("no schedule or tile shape could run this ensemble")
    t, r, sched, b = _parse(min(table, key=table.get))
    if use_cache:
        cache = _load()
        cache[key] = {"threads": t, "rows": r, "schedule": sched, "blocks_per_sm": b, "table": table}
        _store(cache)
    return (t, r, sched, b), table

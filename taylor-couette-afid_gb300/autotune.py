"""Tile-shape autotuner for ensembles.

The launch shape of the grouped kernels -- threads per cell / column / mode
tile and rows per theta-FFT block -- changes no arithmetic (each cell, column,
mode and FFT line is computed by the same device code whatever the tile), so
it can be chosen by timing alone.  ``tune`` builds a scratch ensemble with
the same members, times a few graph replays of every candidate shape and
returns the fastest; the scratch ensemble is then freed, so the runs being
served never advance during tuning.

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


def time_shape(ens, threads: int, rows: int, steps: int) -> float:
    """Seconds per step of `ens` with this tile shape (one warm-up replay,
    which also builds and captures the graph)."""
    ens.tune(threads, rows)
    ens.step(1)
    ens.sync()
    t0 = time.perf_counter()
    ens.step(steps)
    ens.sync()
    return (time.perf_counter() - t0) / steps


def tune(precision: str, bous, states, steps: int = 3, use_cache: bool = True, candidates=None):
    """Best (threads, rows) for an ensemble of these members, and the table
    of measured seconds per step."""
    import tc_gb300 as tc
    key = _device_key() + "|" + signature(precision, bous)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        c = cache[key]
        return (c["threads"], c["rows"]), c.get("table", {})
    cands = candidates or [(t, r) for t in THREADS for r in ROWS]
    ens = tc.Ensemble(precision)
    try:
        for b, s in zip(bous, states):
            ens.add(b, s, dt=1e-6)
        table = {}
        for t, r in cands:
            try:
                table[f"{t}x{r}"] = time_shape(ens, t, r, steps)
            except tc.TCError:
                continue                    # shape not possible for these members
    finally:
        ens.close()
    if not table:
        raise RuntimeError("no tile shape could run this ensemble")
    best = min(table, key=table.get)
    t, r = (int(x) for x in best.split("x"))
    if use_cache:
        cache = _load()
        cache[key] = {"threads": t, "rows": r, "table": table}
        _store(cache)
    return (t, r), table

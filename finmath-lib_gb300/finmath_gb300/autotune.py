"""Autotuner of the portfolio launch: adjoint paths per block, checkpoint stride, products
in flight and Gram blocks per exercise date.

Each candidate records and times the portfolio graph on a subset of the products; the
best configuration is cached in a JSON file keyed by GPU name and problem shape
($FINMATH_GB300_CACHE, default ~/.cache/finmath_gb300/autotune.json).
"""
from __future__ import annotations

import json
import os

DEFAULT = {"adjointThreads": 128, "checkpointStride": 1, "concurrency": 4, "gramBlocks": 0}


def _cache_path():
    base = os.environ.get("FINMATH_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "finmath_gb300"))
    return os.path.join(base, "autotune.json")


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(db, f, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass


def key(gpu_name: str, paths: int, steps: int, periods: int, factors: int, precision: int) -> str:
    return f"v2|{gpu_name}|P{paths}|T{steps}|N{periods}|F{factors}|prec{precision}"


def tune(model, products, cache_key: str, subset: int = 16, force: bool = False, log=None):
    """Return the fastest {adjointThreads, checkpointStride, concurrency, gramBlocks} for this
    problem, measured on `subset` products, cached under cache_key."""
    from .lmm import Portfolio
    db = _load()
    if not force and cache_key in db:
        return dict(db[cache_key]["best"])
    sub = products[:subset]

    def measure(cfg):
        pf = Portfolio(model, sub, True, cfg["checkpointStride"], cfg["concurrency"], cfg["adjointThreads"],
                       cfg["gramBlocks"])
        try:
            pf.run()
            t = min(pf.run()["total_ms"] for _ in range(2))
        finally:
            pf.close()
        if log:
            log(f"autotune {cfg} -> {t:.1f} ms")
        return t

    best = dict(DEFAULT)
    best_t = measure(best)
    trials = [("adjointThreads", [64, 256]), ("checkpointStride", [2, 8]), ("concurrency", [2, 8]),
              ("gramBlocks", [16, 64])]
    results = [(dict(best), best_t)]
    for knob, values in trials:
        for v in values:
            cand = dict(best)
            cand[knob] = v
            t = measure(cand)
            results.append((cand, t))
            if t < best_t:
                best, best_t = cand, t
    db[cache_key] = {"best": best, "best_ms": best_t, "subset": len(sub),
                     "trials": [{"config": c, "ms": t} for c, t in results]}
    _store(db)
    return dict(best)

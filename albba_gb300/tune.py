"""Autotuner: SELL slice height C, sort window sigma, long-row threshold,
block size and the push/pull thresholds (Beamer alpha, beta), picked per
graph-shape class by timing single-root BFS runs on the GPU and cached.

A shape class is (log2 n, log2 mean degree, log2 degree skew), rounded; every
graph of a class reuses the class's entry. The cache is a JSON file next to
this module (tuning/cache.json) keyed by class, holding the chosen
parameters and the timing they were chosen on. The reference fixes
C = 256 and takes sigma from the command line (bfs/src/bfs_SELLCSv2.c:29,
162); it has no tuner.
"""
from __future__ import annotations

import json
import math
import statistics
from pathlib import Path

import numpy as np

import albba_gb300 as ab

CACHE = Path(__file__).resolve().parent / "tuning" / "cache.json"
GRID = {"C": [8, 16, 32, 64], "sigma": [1, 64, 1024, 16384], "block": [128, 256, 512],
        "alpha": [8.0, 14.0, 24.0], "beta": [12.0, 24.0, 48.0], "long_row": [128, 256, 1024]}
DEFAULT = {"C": 32, "sigma": 1024, "long_row": 1024, "block": 256, "alpha": 14.0, "beta": 24.0}


def shape_class(csr: ab.Csr) -> str:
    deg = csr.degrees()
    n = max(csr.n, 1)
    mean = max(float(deg.mean()), 1e-9) if deg.size else 1e-9
    skew = float(deg.max()) / mean if deg.size else 1.0
    return (f"n{round(math.log2(n))}-d{round(math.log2(max(mean, 1.0)))}"
            f"-k{2 * round(math.log2(max(skew, 1.0)) / 2)}")


def _load() -> dict:
    if CACHE.exists():
        try:
            return json.loads(CACHE.read_text())
        except json.JSONDecodeError:
            return {}
    return {}


def _store(cache: dict) -> None:
    CACHE.parent.mkdir(exist_ok=True)
    CACHE.write_text(json.dumps(cache, indent=1, sort_keys=True))


def lookup(csr: ab.Csr) -> dict:
    """Cached parameters for the graph's class, else the defaults."""
    return dict(_load().get(shape_class(csr), {}).get("params", DEFAULT))


def _time(dg: ab.Graph, roots, cfg: dict, repeat: int = 1) -> float:
    opts = ab.bfs_opts("beamer", "graph", alpha=cfg["alpha"], beta=cfg["beta"],
                       block=cfg["block"])
    ms = []
    for _ in range(repeat):
        t = 0.0
        for r in roots:
            t += dg.bfs_device(int(r), None, None, opts).ms
        ms.append(t)
    return statistics.median(ms)


def tune(csr: ab.Csr, roots, grid: dict | None = None, repeat: int = 3) -> dict:
    """Staged search: (C, sigma, long_row), then block, then (alpha, beta)."""
    grid = grid or GRID
    best = dict(DEFAULT)
    best_ms = math.inf
    with ab.Graph(csr, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
        for C_ in grid["C"]:
            for sigma in grid["sigma"]:
                for lr in grid["long_row"]:
                    dg.sell_build(C_, sigma, lr)
                    cfg = dict(best, C=C_, sigma=sigma, long_row=lr)
                    _time(dg, roots[:1], cfg, 1)  # warm-up (graph capture)
                    t = _time(dg, roots, cfg, repeat)
                    if t < best_ms:
                        best, best_ms = cfg, t
        dg.sell_build(best["C"], best["sigma"], best["long_row"])
        for block in grid["block"]:
            cfg = dict(best, block=block)
            _time(dg, roots[:1], cfg, 1)
            t = _time(dg, roots, cfg, repeat)
            if t < best_ms:
                best, best_ms = cfg, t
        for a in grid["alpha"]:
            for b in grid["beta"]:
                cfg = dict(best, alpha=a, beta=b)
                t = _time(dg, roots, cfg, repeat)
                if t < best_ms:
                    best, best_ms = cfg, t
    best["ms"] = best_ms
    return best


def get(csr: ab.Csr, roots, tune_missing: bool = True, grid: dict | None = None) -> dict:
    """Parameters for csr's class: from the cache, or tuned now and cached."""
    cache = _load()
    key = shape_class(csr)
    if key in cache:
        return dict(cache[key]["params"])
    if not tune_missing:
        return dict(DEFAULT)
    res = tune(csr, roots, grid)
    params = {k: res[k] for k in DEFAULT}
    cache[key] = {"params": params, "ms": res["ms"], "n": csr.n, "nnz": csr.nnz,
                  "roots": len(roots)}
    _store(cache)
    return params


def build(csr: ab.Csr, params: dict) -> ab.Graph:
    dg = ab.Graph(csr, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED)
    dg.sell_build(params["C"], params["sigma"], params["long_row"])
    return dg


def worklist_specs(count: int = 256, seed: int = 42) -> list[dict]:
    """The work-list workload: RMAT graphs with scales uniform in 10..18 and
    edge factors from {4, 8, 16, 32}, each with 8 seeded roots."""
    rng = np.random.default_rng(seed)
    return [{"scale": int(rng.integers(10, 19)), "edgefactor": int(rng.choice([4, 8, 16, 32])),
             "seed": 10_000 + i} for i in range(count)]

"""Measurement driver for the workload families beside the headline bench.

  python -m albba_gb300.configs scales   [--scales 20 22 24 26]
  python -m albba_gb300.configs loops    (grid 4096^2 and ER 2^24: host / graph /
                                         persistent level loops, sigma in {1, 256, 4096})
  python -m albba_gb300.configs batched  (64-root batched vs 64 single-root BFS)
  python -m albba_gb300.configs worklist (256 uneven RMAT graphs x 8 roots, tuned)
  python -m albba_gb300.configs selector (learned vs Beamer on held-out RMAT graphs)

Each prints one JSON line per measurement. Graphs are generated from fixed
seeds; GTEPS follows Graph500: undirected edges in the root's component
divided by the traversal time (device events), harmonic mean over roots for
single-root runs, total edges over the batch time for batched runs.
"""
from __future__ import annotations

import argparse
import json
import statistics
import sys
import time

import numpy as np

import albba_gb300 as ab


def emit(d: dict) -> None:
    print(json.dumps(d), flush=True)


def hmean(xs):
    xs = [x for x in xs if x > 0]
    return len(xs) / sum(1.0 / x for x in xs) if xs else 0.0


def plain_runs(dg, roots, opts):
    g = []
    ms = []
    for r in roots:
        st = dg.bfs_device(int(r), None, None, opts)
        g.append(st.edges / 2 / st.ms / 1e6)
        ms.append(st.ms)
    return hmean(g), ms


def batched_timed(dg, roots, d, opts, reps: int = 3):
    """Milliseconds per 64-root BFS into the device buffer d: CUDA events on
    torch's current stream (made the graph's stream) around reps back-to-back
    calls after one warm-up call, the output expansion included. Returns
    (ms, stats of the last call)."""
    import torch
    s = torch.cuda.current_stream()
    dg.set_stream(s.cuda_stream)
    dg.msbfs64_device(roots, d, opts)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        st = dg.msbfs64_device(roots, d, opts)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, st


def cmd_scales(a):
    for sc in a.scales:
        t0 = time.time()
        g = ab.gen_rmat(sc, 16, seed=24)
        roots = g.pick_roots(a.roots, seed=7)
        gen = time.time() - t0
        with ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
            bms = dg.sell_build(32, 1024)
            plain_runs(dg, roots[:2], ab.bfs_opts())
            hm, ms = plain_runs(dg, roots, ab.bfs_opts("beamer", "graph"))
            emit({"config": "plain-scale", "scale": sc, "n": g.n, "stored_entries": g.nnz,
                  "roots": len(roots), "gteps_hmean": hm, "ms_median": statistics.median(ms),
                  "sell_build_ms": bms, "gen_s": gen})
        del g


def cmd_loops(a):
    """Level-loop overhead on high-diameter and low-diameter graphs: every
    loop driver, sigma in {1, 256, 4096}, the Beamer rule and the learned
    selector (when its weights are installed)."""
    from albba_gb300 import selector
    loaded = selector.install()
    policies = ["beamer"] + (["learned"] if loaded.get("plain") else [])
    graphs = [("grid4096", lambda: ab.gen_grid(4096, 4096, 0.1, 1e-4, seed=3)),
              ("er2^24", lambda: ab.gen_er(1 << 24, 8.0, seed=3))]
    for name, mk in graphs:
        g = mk()
        roots = g.pick_roots(a.roots, seed=7)
        with ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
            for sigma in (1, 256, 4096):
                bms = dg.sell_build(32, sigma)
                for pol in policies:
                    for loop in ("host", "graph", "persistent"):
                        opts = ab.bfs_opts(pol, loop)
                        plain_runs(dg, roots[:1], opts)
                        hm, ms = plain_runs(dg, roots, opts)
                        st = dg.bfs_device(int(roots[0]), None, None, opts)
                        emit({"config": "loops", "graph": name, "sigma": sigma, "policy": pol,
                              "loop": loop, "levels": st.num_levels,
                              "ms_median": statistics.median(ms),
                              "us_per_level": 1000 * statistics.median(ms) / st.num_levels,
                              "gteps_hmean": hm, "roots": len(roots), "sell_build_ms": bms})
        del g


def cmd_batched(a):
    import torch
    from albba_gb300 import selector
    selector.install()
    for sc in a.scales:
        g = ab.gen_rmat(sc, 16, seed=24)
        roots = g.pick_roots(64, seed=7)
        with ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
            dg.sell_build(32, 1024)
            d = torch.empty((g.n, 64), dtype=torch.int32, device="cuda")
            plain_runs(dg, roots[:2], ab.bfs_opts())
            t = sum(dg.bfs_device(int(r), None, None, ab.bfs_opts()).ms for r in roots)
            for pol in ("beamer", "learned"):
                ms, st = batched_timed(dg, roots, d, ab.bfs_opts(pol))
                emit({"config": "batched", "scale": sc, "policy": pol, "ms": ms,
                      "gteps": st.edges / 2 / ms / 1e6, "levels": st.num_levels,
                      "plain_64_roots_ms": t, "speedup_vs_plain": t / ms})
        del g


def cmd_worklist(a):
    from albba_gb300 import tune
    specs = tune.worklist_specs(a.graphs)
    wl = ab.Worklist()
    keep = []
    t0 = time.time()
    edges_total = 0
    plain_ms = 0.0
    for sp in specs:
        g = ab.gen_rmat(sp["scale"], sp["edgefactor"], seed=sp["seed"])
        roots = g.pick_roots(8, seed=sp["seed"])
        p = tune.get(g, roots) if a.tune else dict(tune.DEFAULT)
        dg = tune.build(g, p)
        wl.add(dg, roots, p["alpha"], p["beta"])
        opts = ab.bfs_opts("beamer", "graph", alpha=p["alpha"], beta=p["beta"], block=p["block"])
        for r in roots:
            st = dg.bfs_device(int(r), None, None, opts)
            edges_total += st.edges // 2
            plain_ms += st.ms
        keep.append((g, dg))
    setup_s = time.time() - t0
    res = {}
    for block in (128, 256, 512):
        wl.run(block)
        st = wl.run(block)[1]
        res[block] = st.ms
    best = min(res, key=res.get)
    emit({"config": "worklist", "graphs": len(specs), "items": len(specs) * 8,
          "persistent_ms": res, "best_block": best, "gteps": edges_total / res[best] / 1e6,
          "sequential_plain_ms": plain_ms, "speedup_vs_sequential": plain_ms / res[best],
          "tuned": a.tune, "setup_s": setup_s})


def cmd_selector(a):
    """Held-out evaluation of the learned selector: RMAT at the given scales
    (edge factor 16, seed 24, not in the training set) plus a held-out grid
    and Erdos-Renyi graph. Per form: GTEPS with the learned policy and with
    Beamer (device time, same roots), levels compared bit for bit between the
    two, and per-level regret of both against the per-level oracle-best
    variant."""
    import torch
    from albba_gb300 import selector
    loaded = selector.install()
    graphs = [(f"rmat s{sc} ef16", (lambda sc=sc: ab.gen_rmat(sc, 16, seed=24))) for sc in a.scales]
    graphs += [("grid 2048x2048", lambda: ab.gen_grid(2048, 2048, 0.1, 1e-4, seed=77)),
               ("er 2^22 d8", lambda: ab.gen_er(1 << 22, 8.0, seed=77))]
    for name, mk in graphs:
        g = mk()
        roots = g.pick_roots(64, seed=7)
        with ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
            dg.sell_build(32, 1024)
            for form in ("plain", "batched"):
                if not loaded.get(form):
                    emit({"config": "selector", "form": form, "error": "no weights"})
                    continue
                res = {}
                if form == "plain":
                    sub = roots[:a.roots]
                    for pol in ("learned", "beamer"):
                        plain_runs(dg, sub[:1], ab.bfs_opts(pol))
                        res[pol] = plain_runs(dg, sub, ab.bfs_opts(pol))[0]
                    same = all(np.array_equal(dg.bfs(int(r), ab.bfs_opts("learned"))[0],
                                              dg.bfs(int(r), ab.bfs_opts("beamer"))[0])
                               for r in sub[:4])
                else:
                    d = torch.empty((g.n, 64), dtype=torch.int32, device="cuda")
                    out = {}
                    for pol in ("learned", "beamer"):
                        ms, st = batched_timed(dg, roots, d, ab.bfs_opts(pol))
                        res[pol] = st.edges / 2 / ms / 1e6
                        out[pol] = d.cpu().numpy()
                    same = bool(np.array_equal(out["learned"], out["beamer"]))
                    del d
                pr = selector.profile_graph(g, form, min(a.roots, 4), seed=7)
                feat, us, state, group = pr.arrays()
                w = selector.load(form)
                mlp = selector.regret(us, selector.mlp_choices(w, feat))
                beam = selector.regret(us, selector.beamer_choices(state, group, us.argmin(1)))
                emit({"config": "selector", "graph": name, "form": form,
                      "gteps_learned": res["learned"], "gteps_beamer": res["beamer"],
                      "levels_bit_exact": same, "profiled_levels": len(us),
                      "mlp_regret": mlp, "beamer_regret": beam})
        del g


def cmd_spmv(a):
    """fp64 SELL-32-sigma SpMV (alb_sellmat_*) on RMAT graphs with seeded
    values: kernel microseconds and GB/s of 12 bytes per entry + 24 per row."""
    import numpy as np
    import torch
    for sc in a.scales:
        g = ab.gen_rmat(sc, 16, seed=24)
        rng = np.random.default_rng(5)
        with ab.SellMatrix(g.rowptr, g.col, rng.uniform(-1.0, 1.0, g.nnz), 1024) as m:
            dx = torch.from_numpy(rng.standard_normal(g.n)).cuda()
            dy = torch.empty(g.n, dtype=torch.float64, device="cuda")
            for _ in range(3):
                m.spmv_device(dx, dy)
            us = statistics.median(m.spmv_device(dx, dy) for _ in range(20))
            emit({"config": "spmv", "scale": sc, "n": g.n, "entries": g.nnz,
                  "stored_slots": m.stored, "us": us,
                  "gbs": (12 * g.nnz + 24 * g.n) / us / 1e3, "gflops": 2 * g.nnz / us / 1e3})
        del g


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["scales", "loops", "batched", "worklist", "selector", "spmv"])
    ap.add_argument("--scales", type=int, nargs="*", default=[20, 22, 24])
    ap.add_argument("--roots", type=int, default=64)
    ap.add_argument("--graphs", type=int, default=256)
    ap.add_argument("--tune", action="store_true")
    ap.add_argument("--cache", default=None, help="autotuner cache file to use")
    a = ap.parse_args(argv)
    if a.cache:
        from pathlib import Path

        from albba_gb300 import tune
        tune.CACHE = Path(a.cache)
    {"scales": cmd_scales, "loops": cmd_loops, "batched": cmd_batched,
     "worklist": cmd_worklist, "selector": cmd_selector, "spmv": cmd_spmv}[a.what](a)


if __name__ == "__main__":
    sys.exit(main())

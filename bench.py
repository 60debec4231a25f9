#!/usr/bin/env python3
"""Benchmark: GTEPS on RMAT scale 24, edge factor 16, 64 seeded roots.

A step is one pass of the hot path over one batch: BFS from all 64 roots of
the RMAT s24 ef16 graph (A/B/C/D = .57/.19/.19/.05, vertex ids permuted,
symmetrised, self-loops and duplicates removed). The headline form is the
64-root batched BFS driven by the learned direction selector; the plain form
is 64 single-root direction-optimising BFS runs. GTEPS = sum over roots of
the undirected edges in the root's component / step time (Graph500
convention).

  value  device-resident graph and outputs, CUDA events on the launching
         stream around each step
  e2e    the same work through the C ABI with host buffers: graph upload
         (alb_graph_create), SELL build, traversal and the copy of every
         level (and parent) array back to the host, all inside the timer
  roofline  the dominant kernel of the batched step, its bottom-up level:
         algorithmic bytes counted by the kernels themselves (per level, the
         model in include/albba.h) / CUDA-event duration of the level's
         launches, against the measured HBM copy bandwidth (roofline_plain:
         the same for the single-root bottom-up level)
  cpu_baseline  the reference's level loop (C = 256 SELL, pull + sparse-x
         kernels) restated in C with OpenMP, on this host's cores, for a
         bounded sample of roots

--impl reference times only that CPU port (all host threads) on the same
graph and roots. Multi-GPU runs are independent replicas (one process per
GPU, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS RMAT s24 ef16: learned-switch & 64-root batched vs plain; % HBM peak"
SEED_GRAPH, SEED_ROOTS = 24, 7


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--scale", type=int, default=24)
    p.add_argument("--edgefactor", type=int, default=16)
    p.add_argument("--roots", type=int, default=64)
    p.add_argument("--sigma", type=int, default=1024)
    p.add_argument("--long-row", type=int, default=1024,
                   help="rows with more sources are pulled warp-cooperatively, outside the slices")
    p.add_argument("--cpu-roots", type=int, default=1, help="roots timed for the CPU baseline")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-roofline", action="store_true")
    p.add_argument("--loop", choices=["graph", "host", "persistent"], default="graph",
                   help="level loop of both forms (the batched form has graph and host loops; "
                        "host lets a profiler see its kernels)")
    p.add_argument("--out", default=None, help="also write the JSON line to this file")
    return p.parse_args()


def peaks() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler for the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_graph(args):
    import albba_gb300 as ab
    t0 = time.time()
    g = ab.gen_rmat(args.scale, args.edgefactor, seed=SEED_GRAPH)
    roots = g.pick_roots(args.roots, seed=SEED_ROOTS)
    return g, roots, time.time() - t0


def config(args, g, extra=None):
    c = {"workload": f"RMAT scale {args.scale} edgefactor {args.edgefactor}, {args.roots} roots "
                     "(BFS from every root per step)",
         "n": g.n, "stored_entries": g.nnz, "roots": args.roots, "C": 32, "sigma": args.sigma,
         "long_row": args.long_row,
         "graph_seed": SEED_GRAPH, "root_seed": SEED_ROOTS,
         "l2": "inputs larger than L2 (graph > 1 GB vs 129 MB L2); no flush"}
    if extra:
        c.update(extra)
    return c


# ----------------------------------------------------------------- CPU side
# The reference's level loop runs on a SELL-256 matrix with sigma 16384 (its
# defaults, bfs/src/bfs_SELLCSv2.c:29) and splits every level into 8 tasks
# (chunk_size forced to 8, bfs/src/bfs_SELLCSv2.c:214); the CPU port does the
# same, on all host threads (OpenMP).
REF_C, REF_SIGMA, REF_TASKS = 256, 16384, 8


def ref_config(threads: int) -> dict:
    return {"C": REF_C, "sigma": REF_SIGMA, "long_row": None, "tasks_per_level": REF_TASKS,
            "threads": threads,
            "kernels": "pull (bfs_kernel_SELLCS_DFC_bitmap) + sparse-x "
                       "(bfs_kernel_spmspv_SELLCS_DFC_bitmap) restated in C",
            "input": "graph generated by albba_gb300's host generator (CPU only, before "
                     "the timed region); the timed region runs oracle/refalgo.c only"}


def cpu_baseline(g, roots, nroots: int) -> dict:
    import oracle
    ra = oracle.RefAlgo(g.rowptr, g.col, sigma=REF_SIGMA, ntasks=REF_TASKS)
    deg = g.degrees()
    edges, ms = 0, 0.0
    for r in roots[:nroots]:
        counts, bms = ra.run(int(r))
        lv, _, _ = oracle.bfs(g.rowptr, g.col, int(r))
        edges += int(deg[lv >= 0].sum()) // 2
        ms += bms
    ra.close()
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": edges / ms / 1e6, "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{nroots} of {len(roots)} roots, level loop only (SELL-{REF_C} build "
                      f"{ra.conv_ms:.0f} ms excluded, as the reference times it), "
                      f"{REF_TASKS} tasks per level as in the reference",
            "config": ref_config(threads)}


def run_reference(args, rank: int, world: int) -> None:
    if rank != 0:
        return
    g, roots, _ = make_graph(args)
    import oracle
    ra = oracle.RefAlgo(g.rowptr, g.col, sigma=REF_SIGMA, ntasks=REF_TASKS)
    deg = g.degrees()
    comp = {}
    times = []
    edges = 0
    agree = True
    for i in range(args.warmup + args.steps):
        r = int(roots[i % len(roots)])
        counts, bms = ra.run(r)
        if r not in comp:
            lv, _, _ = oracle.bfs(g.rowptr, g.col, r)
            comp[r] = int(deg[lv >= 0].sum()) // 2
            # the loop's per-level frontier sizes against the queue BFS's
            # level sets (the reference's own -v 1 check), outside the timing
            want = np.bincount(lv[lv >= 0]) if (lv >= 0).any() else np.zeros(0, np.int64)
            agree = agree and np.array_equal(np.asarray(counts), want)
        if i >= args.warmup:
            times.append(bms)
            edges += comp[r]
    ms = sum(times)
    v = edges / ms / 1e6
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"metric": METRIC, "value": v, "unit": "GTEPS", "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / max(len(times), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic RMAT (seeded), reference level loop restated in C (OpenMP)",
            "config": config(args, g, {"step": "one root per step (bounded CPU sample)",
                                       **ref_config(threads)}),
            "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} timed roots, one per step, level loop "
                                       f"only, {REF_TASKS} tasks per level"},
            "frontier_counts_match_oracle": bool(agree),
            "e2e": {"value": v, "unit": "GTEPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    ra.close()
    emit(line, args)


# ----------------------------------------------------------------- GPU side
def timed(stream, fn, steps, sync, dist, torch):
    """CUDA events on the launching stream around `steps` calls of fn (max over ranks)."""
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sync()
    torch.cuda.synchronize()
    ev0.record(stream)
    out = [fn() for _ in range(steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    sync()
    ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, out


def run_ours(args, rank: int, world: int, dist) -> None:
    import torch

    import albba_gb300 as ab
    from albba_gb300 import selector
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    loaded = selector.install()
    g, roots, gen_s = make_graph(args)
    stream = torch.cuda.current_stream()
    dg = ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED)
    dg.set_stream(stream.cuda_stream)
    build_ms = dg.sell_build(32, args.sigma, args.long_row)
    n = g.n
    d_lv = torch.empty(n, dtype=torch.int32, device="cuda")
    d_pa = torch.empty(n, dtype=torch.int32, device="cuda")
    d_ms = torch.empty((n, 64), dtype=torch.int32, device="cuda")
    policy = "learned" if loaded.get("batched") else "beamer"
    bopts = ab.bfs_opts(policy, args.loop)
    popts = ab.bfs_opts("learned" if loaded.get("plain") else "beamer", args.loop)
    sync = (lambda: dist.barrier()) if dist else (lambda: None)

    def batched_step():
        st = dg.msbfs64_device(roots, d_ms, bopts)
        return st.edges // 2, st.kernels

    def plain_step():
        e = k = 0
        per = []
        for r in roots:
            st = dg.bfs_device(int(r), d_lv, d_pa, popts)
            e += st.edges // 2
            k += st.kernels
            per.append((st.edges // 2, st.ms))
        return e, k, per

    for _ in range(args.warmup):
        batched_step()
        plain_step()
    # clocks are sampled across both timed regions (the batched one alone is
    # shorter than the 200 ms sampling interval)
    with Clocks(dev) as clk:
        ms, outs = timed(stream, batched_step, args.steps, sync, dist, torch)
        pms, pouts = timed(stream, plain_step, args.steps, sync, dist, torch)
    edges = sum(e for e, _ in outs)
    launches = sum(k for _, k in outs)
    value = world * edges / ms / 1e6
    pedges = sum(o[0] for o in pouts)
    per_root = [x for o in pouts for x in o[2]]
    plain = world * pedges / pms / 1e6
    hm = len(per_root) / sum(m / (e / 1e6) for e, m in per_root if e > 0) if per_root else None

    # the end-to-end steps first, while the memory pool holds only the
    # bench's own graph (the measurements below allocate and free more)
    e2e = None if args.no_e2e else e2e_batched(args, g, roots, ab, torch, bopts)
    roof = None if args.no_roofline else roofline(dg, roots, d_ms, policy)
    roof_plain = None if args.no_roofline else roofline_plain(dg, roots[:8])
    heldout = selector_heldout(dg, g, roots, loaded)
    spmv = None if args.no_roofline else spmv_roofline(g)
    cpu = cpu_baseline(g, roots, args.cpu_roots) if rank == 0 and args.cpu_roots > 0 else None
    if rank != 0:
        return
    meta = {f: (json.loads((selector.WEIGHTS / f"{f}.json").read_text()).get("meta", {})
                if loaded.get(f) else None) for f in ("plain", "batched")}
    line = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic RMAT (seeded generator, no dataset)",
            "config": config(args, g, {
                "form": f"64-root bit-parallel batched BFS, {policy} direction selector",
                "parallelism": f"replicas x{world}"}),
            "plain": {"gteps": plain, "gteps_harmonic_mean": hm, "ms_per_step": pms / args.steps,
                      "form": "64 single-root direction-optimising BFS "
                              f"({'learned' if loaded.get('plain') else 'beamer'}, {args.loop} loop)"},
            "batched_over_plain": value / plain if plain else None,
            "selector": {"batched": policy, "weights": {f: bool(loaded.get(f)) for f in loaded},
                         "heldout_measured": heldout,
                         "heldout_at_training": {f: (m or {}).get("heldout")
                                                 for f, m in meta.items()}},
            "sell_build_ms": build_ms, "graph_gen_s": gen_s,
            "gpu_launches": launches, "clocks": clk.summary(), "roofline": roof,
            "roofline_plain": roof_plain, "spmv": spmv,
            "e2e": e2e, "cpu_baseline": cpu}
    emit(line, args)


def roofline(dg, roots, d_ms, policy) -> dict:
    """Dominant kernel of the batched step: the bottom-up level of the 64-root
    BFS (k_ms_bu over the slices, then the long-row head/tail passes and their
    fold-in, the push of the pushed roots and the frontier sampling). Bytes
    are counted by the kernels themselves (the model in include/albba.h); time
    is CUDA events around the level's launches on the graph's stream, from the
    host-driven trace run with the bench's policy."""
    import albba_gb300 as ab
    peak, kind = peaks()
    byts, us, nlev = 0, 0.0, 0
    for _ in range(2):  # the first run warms the trace path
        dg.msbfs64_device(roots, d_ms, ab.bfs_opts(policy, trace=True))
    per_level = []
    for t in dg.level_trace():
        if t.dir != ab.DIR_TOPDOWN and t.step_us > 0:
            byts += t.bytes
            us += t.step_us
            nlev += 1
            per_level.append({"level": t.level, "bytes": t.bytes, "us": round(t.step_us, 1),
                              "gbs": round(t.bytes / t.step_us / 1e3, 1)})
    gbs = byts / us / 1e3 if us > 0 else 0.0
    return {"bound": "hbm",
            "kernel": "k_ms_bu + k_ms_bu_long + k_ms_bu_long_tail + k_ms_bu_long_fin "
                      "+ k_ms_tq + k_ms_td<push> + k_ms_td_big<push> + k_ms_sample "
                      "(64-root bottom-up level)",
            "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_kind": f"{kind} HBM copy bandwidth (burst)",
            "bytes_per_launch": byts / max(nlev, 1), "us_per_launch": us / max(nlev, 1),
            "launches": nlev, "levels": per_level,
            # DRAM bytes need an ncu capture, which this run does not take
            # (one-kernel captures of a smaller graph are summarised under
            # profiles/)
            "traffic": None}


def selector_heldout(dg, g, roots, loaded, plain_roots: int = 4) -> dict:
    """The selector's per-level regret on this run's graph, measured here:
    every level of the traversal is run with each of the three variants from
    the same state and timed (alb_msbfs64_profile / alb_bfs_profile); the
    regret of a rule is its choices' time over the fastest variant's. The
    networks were trained on other graphs, so this graph is held out."""
    import albba_gb300 as ab
    from albba_gb300 import selector
    out = {"graph": "this run's graph (held out from training)"}
    for form in ("batched", "plain"):
        if not loaded.get(form):
            continue
        prof = selector.Profiles()
        if form == "batched":
            prof.add(dg.msbfs64_profile(roots, ab.bfs_opts("beamer")), g.n, 0)
        else:
            for i, r in enumerate(roots[:plain_roots]):
                prof.add(dg.bfs_profile(int(r), ab.bfs_opts("beamer", "host")), g.n, i)
        feat, us, state, group = prof.arrays()
        best = us.argmin(axis=1)
        w = selector.load(form)
        out[form] = {"levels": int(len(us)),
                     "roots": len(roots) if form == "batched" else min(plain_roots, len(roots)),
                     "mlp": selector.regret(us, selector.mlp_choices(w, feat)),
                     "beamer": selector.regret(us, selector.beamer_choices(state, group, best))}
    return out


def spmv_roofline(g, reps: int = 20) -> dict:
    """The fp64 SELL-C-sigma SpMV (alb_sellmat_spmv, the reference's
    kernel_SELLCS_DFC) on this run's graph with seeded values: algorithmic
    bytes per launch = 12 per stored entry (int32 column + fp64 value) +
    24 per row (x read once, y written, row order and length read) over the
    kernel's CUDA-event time, against the measured HBM copy bandwidth.
    Bit-exact y keeps every row's fma chain in CSR order, so no launch ends
    before the longest row's chain: that row alone (the same entries, every
    other row empty) is timed the same way as the launch's latency floor."""
    import torch

    import albba_gb300 as ab
    peak, kind = peaks()
    rng = np.random.default_rng(5)
    val = rng.uniform(-1.0, 1.0, g.nnz)
    x = rng.standard_normal(g.n)

    def median_us(rp, col, v):
        with ab.SellMatrix(rp, col, v, 1024) as m:
            dx = torch.from_numpy(x).cuda()
            dy = torch.empty(g.n, dtype=torch.float64, device="cuda")
            for _ in range(3):
                m.spmv_device(dx, dy)
            return statistics.median(m.spmv_device(dx, dy) for _ in range(reps)), m.stored

    t, stored = median_us(g.rowptr, g.col, val)
    deg = np.diff(g.rowptr)
    r = int(deg.argmax())
    lo, hi = int(g.rowptr[r]), int(g.rowptr[r + 1])
    rp1 = np.zeros(g.n + 1, np.int64)
    rp1[r + 1:] = hi - lo
    t_floor, _ = median_us(rp1, g.col[lo:hi], val[lo:hi])
    byts = 12 * g.nnz + 24 * g.n
    gbs = byts / t / 1e3
    return {"kernel": "k_spmv + k_spmv_long (fp64 SELL-32-sigma SpMV, y = A x)",
            "bound": "the longest row's dependent fp64 fma chain (bit-exact order)",
            "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_kind": f"{kind} HBM copy bandwidth (burst)", "bytes_per_launch": byts,
            "us_per_launch": t, "stored_slots": stored, "entries": g.nnz,
            "gflops": 2 * g.nnz / t / 1e3,
            "latency_floor": {"longest_row": hi - lo, "us": t_floor,
                              "ns_per_entry": 1e3 * t_floor / max(hi - lo, 1),
                              "launch_over_floor": t / t_floor if t_floor > 0 else None}}


def roofline_plain(dg, roots) -> dict:
    """Bottom-up level of the single-root BFS (k_bu_long, k_bu_long_tail,
    k_bu), same method, host-driven loop with the Beamer rule."""
    import albba_gb300 as ab
    peak, kind = peaks()
    byts, us, nlev = 0, 0.0, 0
    for r in roots:
        dg.bfs(int(r), ab.bfs_opts("beamer", "host", trace=True), want_level=False,
               want_parent=False)
        for t in dg.level_trace():
            if t.dir != ab.DIR_TOPDOWN and t.step_us > 0:
                byts += t.bytes
                us += t.step_us
                nlev += 1
    gbs = byts / us / 1e3 if us > 0 else 0.0
    return {"kernel": "k_bu_long + k_bu_long_tail + k_bu (single-root bottom-up level)",
            "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "bytes_per_launch": byts / max(nlev, 1), "us_per_launch": us / max(nlev, 1),
            "launches": nlev, "roots": len(roots)}


def copy_floor(torch, nbytes: int = 1 << 30) -> dict:
    """Page-locked host <-> device copy bandwidth on this machine (CUDA events,
    best of 5 copies of 1 GiB each way): the floor under e2e's copies."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = None
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            dst.copy_(src, non_blocking=True)
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = nbytes / best / 1e6
    del h, d
    return out


def e2e_batched(args, g, roots, ab, torch, opts, steps: int = 10) -> dict:
    """Host CSR in, host levels out, through the C ABI: alb_graph_create +
    alb_sell_build + alb_msbfs64 (n x 64 int32 levels copied back)."""
    # page-locked host buffers: the graph the caller hands over and the levels
    # it gets back (filled once, before the timed region)
    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    rp = pinned((g.n + 1,), torch.int64)
    rp[:] = g.rowptr
    col = pinned((g.col.shape[0],), torch.int32)
    col[:] = g.col
    hg = ab.Csr(rp, col)
    levels = pinned((g.n, 64), torch.int32)
    h2d = rp.nbytes + col.nbytes
    d2h = levels.nbytes
    flags = ab.CSR_SYMMETRIC | ab.CSR_SORTED

    def step():
        with ab.Graph(hg, flags=flags) as dg:
            dg.sell_build(32, args.sigma, args.long_row)
            ab.check(ab.lib().alb_msbfs64(dg.handle, roots.ctypes.data, len(roots),
                                          ab.C.byref(opts), levels.ctypes.data,
                                          ab.C.byref(ab.Stats())))
        return 0

    # two untimed steps first: the host<->device link and the memory pool
    # reach their steady state (the first copies after the host has been
    # busy run several times slower)
    for _ in range(2):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    marks = []
    for _ in range(steps):
        step()  # returns after the levels are in host memory
        marks.append(time.perf_counter())
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    per_step = [(b - a) * 1e3 for a, b in zip([t0] + marks[:-1], marks)]
    # phase split of one more step, right away (wall clock, a synchronize
    # after each call)
    ph = {}
    t = time.perf_counter()
    dg = ab.Graph(hg, flags=flags)
    torch.cuda.synchronize()
    ph["graph_create_ms"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    dg.sell_build(32, args.sigma, args.long_row)
    torch.cuda.synchronize()
    ph["sell_build_ms"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    ab.check(ab.lib().alb_msbfs64(dg.handle, roots.ctypes.data, len(roots), ab.C.byref(opts),
                                  levels.ctypes.data, ab.C.byref(ab.Stats())))
    torch.cuda.synchronize()
    ph["msbfs64_with_level_copy_ms"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    dg.close()
    torch.cuda.synchronize()
    ph["graph_destroy_ms"] = (time.perf_counter() - t) * 1e3
    deg = g.degrees()
    edges = 0
    for i in range(len(roots)):
        edges += int(deg[levels[:, i] >= 0].sum()) // 2
    fl = copy_floor(torch)
    floor_ms = h2d / fl["h2d_gbs"] / 1e6 + d2h / fl["d2h_gbs"] / 1e6
    return {"value": steps * edges / dt / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": steps, "ms_per_step": dt / steps * 1e3,
            "step_ms": [round(x, 2) for x in per_step],
            "phases": {k: round(v, 2) for k, v in ph.items()},
            "copy_floor": {"h2d_gbs": round(fl["h2d_gbs"], 1), "d2h_gbs": round(fl["d2h_gbs"], 1),
                           "ms_per_step": round(floor_ms, 2),
                           "how": "page-locked 1 GiB copies, best of 5, CUDA events"},
            "path": "alb_graph_create (host CSR) + alb_sell_build + alb_msbfs64 (host n x 64 "
                    "levels), wall clock"}


def emit(line: dict, args) -> None:
    s = json.dumps(line)
    print(s, flush=True)
    if args.out:
        Path(args.out).write_text(s + "\n")


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        td.init_process_group("nccl")
        dist = td
    run_ours(args, rank, world, dist)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

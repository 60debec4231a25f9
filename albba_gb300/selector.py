"""Learned direction selector: data collection, GPU training, evaluation.

Per level the selector picks one of three traversal variants (top-down push,
bottom-up pull with bypass, bottom-up pull without bypass). Its training
data are per-level oracle timings: alb_bfs_profile / alb_msbfs64_profile run
every variant from the same state and time each with CUDA events. The
network (8 -> 32 -> 32 -> 3, ReLU, fp32) regresses log2 of each variant's
step time; the cheapest prediction wins. Training runs on the GPU through the
library's own forward/backward/Adam kernels (alb_selector_train). The Beamer
alpha/beta rule stays as the fallback when no weights are loaded.

Weights are stored as JSON next to this file (selector_weights/plain.json for the
single-root BFS, selector_weights/batched.json for the 64-root batched BFS) with the
metadata of the run that produced them.

The reference (scalbba/albba) switches kernels on a fixed frontier-size
threshold (bfs/src/bfs_SELLCSv2.c:283-284); the learned selector has no
counterpart there.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

import albba_gb300 as ab

WEIGHTS = Path(__file__).resolve().parent / "selector_weights"
FORMS = {"plain": 0, "batched": 1}


# ------------------------------------------------------------------ graphs
def training_specs(full: bool = False, seed: int = 0) -> list[dict]:
    """Graph specs for training. full=True: 400 graphs (RMAT scales 16-24,
    edge factors 4-64, plus grid and Erdos-Renyi families); otherwise a
    reduced set of the same families at scales 14-21 that profiles in a few
    minutes."""
    rng = np.random.default_rng(seed)
    specs = []
    if full:
        for i in range(360):
            specs.append({"kind": "rmat", "scale": int(rng.integers(16, 25)),
                          "edgefactor": int(rng.choice([4, 8, 16, 32, 64])), "seed": 1000 + i})
        for i in range(20):
            side = int(rng.choice([1024, 2048, 4096]))
            specs.append({"kind": "grid", "rows": side, "cols": side, "drop": 0.1,
                          "shortcut_frac": 1e-4, "seed": 2000 + i})
        for i in range(20):
            specs.append({"kind": "er", "n": int(2 ** rng.integers(18, 25)), "mean_degree": 8.0,
                          "seed": 3000 + i})
        return specs
    for i, (sc, ef) in enumerate([(14, 4), (14, 32), (15, 16), (16, 8), (16, 64), (17, 4),
                                  (17, 16), (18, 32), (18, 8), (19, 16), (19, 64), (20, 4),
                                  (20, 16), (20, 32), (21, 8), (21, 16)]):
        specs.append({"kind": "rmat", "scale": sc, "edgefactor": ef, "seed": 1000 + i})
    specs.append({"kind": "grid", "rows": 512, "cols": 512, "drop": 0.1, "shortcut_frac": 1e-4,
                  "seed": 2000})
    specs.append({"kind": "grid", "rows": 1024, "cols": 1024, "drop": 0.1, "shortcut_frac": 1e-4,
                  "seed": 2001})
    specs.append({"kind": "er", "n": 1 << 19, "mean_degree": 8.0, "seed": 3000})
    specs.append({"kind": "er", "n": 1 << 21, "mean_degree": 8.0, "seed": 3001})
    return specs


def make_graph(spec: dict) -> ab.Csr:
    k = spec["kind"]
    if k == "rmat":
        return ab.gen_rmat(spec["scale"], spec["edgefactor"], spec["seed"])
    if k == "grid":
        return ab.gen_grid(spec["rows"], spec["cols"], spec["drop"], spec["shortcut_frac"],
                           spec["seed"])
    return ab.gen_er(spec["n"], spec["mean_degree"], spec["seed"])


# ------------------------------------------------------------------ data
@dataclass
class Profiles:
    feat: list = field(default_factory=list)   # [N, 8]
    us: list = field(default_factory=list)     # [N, 3]
    state: list = field(default_factory=list)  # [N, 6]: level, nf, mf, nu, mu, n
    group: list = field(default_factory=list)  # traversal id per level

    def add(self, recs, n: int, gid: int) -> None:
        for p in recs:
            self.feat.append(list(p.feat))
            self.us.append(list(p.us))
            self.state.append([p.rec.level, p.rec.nf, p.rec.mf, p.rec.nu, p.rec.mu, n])
            self.group.append(gid)

    def arrays(self):
        return (np.array(self.feat, np.float32), np.array(self.us, np.float32),
                np.array(self.state, np.float64), np.array(self.group, np.int64))

    def extend(self, other: "Profiles") -> None:
        off = (max(self.group) + 1) if self.group else 0
        self.feat += other.feat
        self.us += other.us
        self.state += other.state
        self.group += [g + off for g in other.group]


def profile_graph(csr: ab.Csr, form: str, nroots: int, seed: int = 5, C_: int = 32,
                  sigma: int = 1024, max_levels: int = 200) -> Profiles:
    out = Profiles()
    roots = csr.pick_roots(nroots if form == "plain" else 64, seed)
    with ab.Graph(csr, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
        dg.sell_build(C_, sigma)
        if form == "plain":
            for i, r in enumerate(roots[:nroots]):
                recs = dg.bfs_profile(int(r), ab.bfs_opts("beamer", "host"))
                out.add(_thin(recs, max_levels), csr.n, i)
        else:
            recs = dg.msbfs64_profile(roots, ab.bfs_opts("beamer"))
            out.add(_thin(recs, max_levels), csr.n, 0)
    return out


def _thin(recs, max_levels):
    # long-diameter traversals (grids) would dominate the set: keep an even sample
    if len(recs) <= max_levels:
        return recs
    idx = np.linspace(0, len(recs) - 1, max_levels).astype(int)
    return [recs[i] for i in idx]


def targets(us: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    y = np.log2(np.maximum(us, 1.0)).astype(np.float32)
    return y, np.ones_like(y, dtype=np.float32)


# ------------------------------------------------------------- train / eval
def train(feat, us, steps: int = 4000, lr: float = 3e-3, seed: int = 0):
    y, m = targets(us)
    return ab.selector_train(feat, y, m, steps=steps, lr=lr, seed=seed)


def mlp_choices(params, feat) -> np.ndarray:
    return np.argmin(ab.mlp_forward(params, feat), axis=1)


def beamer_choices(state: np.ndarray, group: np.ndarray, best: np.ndarray,
                   alpha: float = 14.0, beta: float = 24.0) -> np.ndarray:
    """The Beamer rule of the library (dev.cuh beamer_dir) replayed on profiled
    levels; the previous direction is the variant the profile run took."""
    out = np.zeros(len(state), np.int64)
    for i, (lvl, nf, mf, nu, mu, n) in enumerate(state):
        first = i == 0 or group[i] != group[i - 1]
        prev_dir = -1 if first else int(best[i - 1])
        prev_nf = 0 if first else state[i - 1][1]
        if prev_dir < 0 or prev_dir == ab.DIR_TOPDOWN:
            out[i] = ab.DIR_BOTTOMUP if mf > mu / alpha else ab.DIR_TOPDOWN
        else:
            stay = nf >= prev_nf or nf > n / beta
            out[i] = ab.DIR_BOTTOMUP if stay else ab.DIR_TOPDOWN
    return out


def regret(us: np.ndarray, choice: np.ndarray) -> dict:
    best = us.min(axis=1)
    chosen = us[np.arange(len(us)), choice]
    return {"total": float(chosen.sum() / best.sum() - 1.0),
            "mean_level": float(np.mean(chosen / best - 1.0)),
            "median_level": float(np.median(chosen / best - 1.0)),
            "chosen_us": float(chosen.sum()), "best_us": float(best.sum())}


def save(params: np.ndarray, form: str, meta: dict, out_dir: Path | None = None) -> Path:
    d = Path(out_dir) if out_dir else WEIGHTS
    d.mkdir(parents=True, exist_ok=True)
    p = d / f"{form}.json"
    p.write_text(json.dumps({"form": form, "nparam": int(params.size),
                             "params": [float(x) for x in params], "meta": meta}))
    return p


def load(form: str) -> np.ndarray | None:
    p = WEIGHTS / f"{form}.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return np.array(d["params"], np.float32)


def install(forms=("plain", "batched")) -> dict:
    """Load stored weights into the library (selector 0 = plain, 1 = batched)."""
    done = {}
    for f in forms:
        w = load(f)
        if w is not None:
            ab.selector_load(FORMS[f], w)
        done[f] = w is not None
    return done


def run(full: bool, forms, roots: int, steps: int, heldout_scale: int, log=print,
        out_dir: Path | None = None) -> dict:
    report = {}
    specs = training_specs(full)
    # every graph is generated once and profiled for every form; the host
    # generates the next graph while the GPU profiles the current one
    t0 = time.time()
    datas = {form: Profiles() for form in forms}
    with ThreadPoolExecutor(max_workers=1) as pool:
        nxt = pool.submit(make_graph, specs[0]) if specs else None
        for i, spec in enumerate(specs):
            csr = nxt.result()
            nxt = pool.submit(make_graph, specs[i + 1]) if i + 1 < len(specs) else None
            for form in forms:
                datas[form].extend(profile_graph(csr, form, roots, seed=11 + i))
            del csr
            if (i + 1) % 25 == 0:
                print(f"profiled {i + 1}/{len(specs)} graphs in {time.time() - t0:.0f} s",
                      file=sys.stderr, flush=True)
    t1 = time.time()
    for form in forms:
        feat, us, state, group = datas[form].arrays()
        tf = time.time()
        params, loss = train(feat, us, steps=steps)
        t2 = time.time()
        best = us.argmin(axis=1)
        tr = {"mlp": regret(us, mlp_choices(params, feat)),
              "beamer": regret(us, beamer_choices(state, group, best))}
        # held-out graph
        ho = make_graph({"kind": "rmat", "scale": heldout_scale, "edgefactor": 16, "seed": 24})
        hp = profile_graph(ho, form, roots, seed=7)
        hf, hus, hst, hgr = hp.arrays()
        hb = hus.argmin(axis=1)
        held = {"mlp": regret(hus, mlp_choices(params, hf)),
                "beamer": regret(hus, beamer_choices(hst, hgr, hb))}
        meta = {"graphs": len(specs), "full_spec": full, "levels": int(len(us)),
                "train_loss": loss, "steps": steps, "profile_s": t1 - t0, "train_s": t2 - tf,
                "train_regret": tr, "heldout": {"graph": f"rmat s{heldout_scale} ef16",
                                                "regret": held}}
        save(params, form, meta, out_dir)
        report[form] = meta
        log(json.dumps({form: meta}))
    return report


def main():
    ap = argparse.ArgumentParser(description="profile, train and store the direction selector")
    ap.add_argument("--full", action="store_true", help="400-graph training set")
    ap.add_argument("--forms", default="plain,batched")
    ap.add_argument("--roots", type=int, default=4)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--heldout-scale", type=int, default=22)
    ap.add_argument("--out-dir", default=None, help="where to write <form>.json")
    a = ap.parse_args()
    run(a.full, a.forms.split(","), a.roots, a.steps, a.heldout_scale, out_dir=a.out_dir)


if __name__ == "__main__":
    main()

"""Generate tests/golden/*.json from the reference's own code.

Builds oracle/_ref/libalbba_ref.so from the reference sources (read in place,
unchanged; see oracle/Makefile.ref) and records, for small seeded graphs:

  * bfs_counts.json  per-level frontier sizes of the reference's verifier
    run_bfs_ref (bfs/src/bfs_ref.h:26-67) for several roots. The reference
    always starts at row 0, so each root is moved to row 0 by swapping the
    labels 0 <-> root (level sizes do not depend on labels);
  * sell.json        row_order / slice_widths / slice_pointers and a checksum
    of the padded column layout from get_order_by_row_size_radix +
    convert_csr_to_sellcs (bfs/src/sorting_utils.c:232-253,
    bfs/src/sparse_matrix.c:435-521), plus the full layout of one tiny graph;
  * custom_bfs.json  per-level frontier sizes of the reference's own level
    loop run_custom_bfs_test (bfs/src/bfs_SELLCSv2.c:126-820) with its VE
    kernels restated in scalar C (oracle/ref/ve_scalar.c).

Graphs come from the albba_gb300 generators (deterministic in their
parameters); each record stores the parameters and a checksum of the graph.

Run:  python tests/golden/make_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import albba_gb300 as ab  # noqa: E402
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent

GRAPHS = [
    {"kind": "rmat", "scale": 10, "edgefactor": 16, "seed": 11},
    {"kind": "rmat", "scale": 12, "edgefactor": 8, "seed": 12},
    {"kind": "rmat", "scale": 12, "edgefactor": 16, "seed": 13},
    {"kind": "grid", "rows": 48, "cols": 40, "drop": 0.1, "shortcut_frac": 0.002, "seed": 14},
    {"kind": "er", "n": 3000, "mean_degree": 4.0, "seed": 15},
    {"kind": "tiny", "name": "path_star"},
]


def tiny_graph(name: str) -> ab.Csr:
    # a path 0-1-2-3-4, a star centred at 5 with leaves 6..9 linked to 4,
    # an isolated vertex 10 and a separate edge 11-12
    u = [0, 1, 2, 3, 5, 5, 5, 5, 4, 11]
    v = [1, 2, 3, 4, 6, 7, 8, 9, 9, 12]
    return ab.csr_from_edges(13, np.array(u), np.array(v))


def make_graph(spec: dict) -> ab.Csr:
    k = spec["kind"]
    if k == "rmat":
        return ab.gen_rmat(spec["scale"], spec["edgefactor"], spec["seed"])
    if k == "grid":
        return ab.gen_grid(spec["rows"], spec["cols"], spec["drop"], spec["shortcut_frac"],
                           spec["seed"])
    if k == "er":
        return ab.gen_er(spec["n"], spec["mean_degree"], spec["seed"])
    return tiny_graph(spec["name"])


def checksum(g: ab.Csr) -> int:
    rp = g.rowptr.astype(np.uint64)
    col = g.col.astype(np.uint64)
    idx = np.arange(col.shape[0], dtype=np.uint64)
    return int((np.sum(rp * np.uint64(2654435761)) + np.sum((col + np.uint64(1)) * (idx % np.uint64(1009) + np.uint64(1)))) % np.uint64(2**61 - 1))


def relabel(g: ab.Csr, root: int):
    """int32 CSR with labels 0 and root swapped, rows ascending."""
    n = g.n
    pi = np.arange(n, dtype=np.int64)
    pi[0], pi[root] = root, 0
    deg = np.diff(g.rowptr)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    ns, nd = pi[src], pi[g.col.astype(np.int64)]
    order = np.lexsort((nd, ns))
    ns, nd = ns[order], nd[order]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, ns + 1, 1)
    rp = np.cumsum(rp)
    return rp.astype(np.int32), nd.astype(np.int32)


def main() -> None:
    if oracle.build_reference() is None:
        sys.exit("reference tree not found")
    R = oracle.ref_lib()
    bfs_recs, sell_recs, custom_recs = [], [], []
    for spec in GRAPHS:
        g = make_graph(spec)
        n = g.n
        roots = [0] if spec["kind"] == "tiny" else g.pick_roots(6, 99).tolist()
        if spec["kind"] == "tiny":
            roots = [0, 5, 10, 11]
        for root in roots:
            rp, col = relabel(g, int(root))
            counts = np.zeros(n + 1, np.int32)
            nl = R.refh_bfs_counts(n, rp.ctypes.data, col.ctypes.data, counts.ctypes.data)
            bfs_recs.append({"graph": spec, "checksum": checksum(g), "n": n, "nnz": g.nnz,
                             "root": int(root), "counts": counts[:nl].tolist()})
            if spec["kind"] != "tiny":
                for sigma in (256, 16384):
                    fr = np.zeros(n + 1, np.int32)
                    nv, dead = np.zeros(1, np.int32), np.zeros(1, np.int32)
                    ni = R.refh_custom_bfs(n, rp.ctypes.data, col.ctypes.data, sigma,
                                           fr.ctypes.data, nv.ctypes.data, dead.ctypes.data)
                    custom_recs.append({"graph": spec, "checksum": checksum(g), "root": int(root),
                                        "sigma": sigma, "counts": fr[:ni].tolist(),
                                        "num_vex": int(nv[0]), "dead_calls": int(dead[0]),
                                        "matches_run_bfs_ref": fr[:ni].tolist() == counts[:nl].tolist()})
        rp32 = g.rowptr.astype(np.int32)
        col32 = np.ascontiguousarray(g.col, dtype=np.int32)
        for C_, sigma in ((8, 8), (16, 64), (32, 32), (32, 1024), (64, 64), (64, 16384), (256, 16384)):
            if spec["kind"] == "tiny" and C_ > 16:
                continue
            ns = (n + C_ - 1) // C_
            total = R.refh_sell(n, rp32.ctypes.data, col32.ctypes.data, C_, sigma, None, None, None, None)
            order = np.zeros(n, np.int32)
            widths = np.zeros(ns, np.int32)
            sptr = np.zeros(ns + 1, np.int32)
            pcol = np.zeros(max(total, 1), np.int32)
            R.refh_sell(n, rp32.ctypes.data, col32.ctypes.data, C_, sigma, order.ctypes.data,
                        widths.ctypes.data, sptr.ctypes.data, pcol.ctypes.data)
            rec = {"graph": spec, "checksum": checksum(g), "C": C_, "sigma": sigma,
                   "row_order": order.tolist(), "slice_widths": widths.tolist(),
                   "slice_pointers": sptr.tolist(),
                   "padded_col_sum": int(np.sum(pcol[:total].astype(np.int64) *
                                               (np.arange(total, dtype=np.int64) % 7919 + 1)))}
            if spec["kind"] == "tiny":
                rec["padded_col"] = pcol[:total].tolist()
            sell_recs.append(rec)
        # active-lane ("DFC") layout at C = 256 for the CPU port of the reference
        nops = R.refh_sell_dfc(n, rp32.ctypes.data, col32.ctypes.data, 16384, None, None)
        if spec["kind"] != "tiny":
            vl = np.zeros(max(nops, 1), np.int32)
            sp = np.zeros((n + 255) // 256 + 1, np.int32)
            R.refh_sell_dfc(n, rp32.ctypes.data, col32.ctypes.data, 16384, vl.ctypes.data, sp.ctypes.data)
            sell_recs.append({"graph": spec, "checksum": checksum(g), "C": 256, "sigma": 16384,
                              "dfc": True, "vop_lengths_sum": int(vl[:nops].astype(np.int64).sum()),
                              "nops": int(nops), "slice_pointers": sp.tolist()})
    (OUT / "bfs_counts.json").write_text(json.dumps(bfs_recs, separators=(",", ":")))
    (OUT / "sell.json").write_text(json.dumps(sell_recs, separators=(",", ":")))
    (OUT / "custom_bfs.json").write_text(json.dumps(custom_recs, indent=0, separators=(",", ":")))
    mism = sum(not r["matches_run_bfs_ref"] for r in custom_recs)
    print(f"{len(bfs_recs)} bfs records, {len(sell_recs)} sell records, "
          f"{len(custom_recs)} custom-loop records ({mism} differ from run_bfs_ref)")


if __name__ == "__main__":
    main()

"""Parity at the benchmarked configuration.

The bench times the 64-root batched BFS on RMAT scale 24, edge factor 16
(graph seed 24, root seed 7), SELL-32 with sigma 1024 and long rows over
1024, driven by the shipped learned selector in the CUDA-graph level loop
with the default push budget for small-frontier roots. Here that exact form
runs once and every root's levels are compared with the single-root BFS of
the same root (itself checked against the oracle, the CPU restatement of
the reference verifier run_bfs_ref, bfs/src/bfs_ref.h:26-67), four roots
directly against the oracle, and their parents against the oracle's
smallest-parent rule and the BFS validator. Scale 26 runs once as well, at
edge factor 17: its 2.2 G stored entries put row offsets past 2^31, which
the reference's int CSR (bfs/src/sparse_matrix.h:26) cannot hold (at edge
factor 16 the symmetrised graph keeps 2.10 G entries, just under 2^31)."""
from __future__ import annotations

import numpy as np
import pytest

import albba_gb300 as ab
import oracle
from albba_gb300 import selector

pytestmark = pytest.mark.gpu


@pytest.fixture
def learned_weights():
    loaded = selector.install()
    yield loaded
    ab.selector_clear(0)
    ab.selector_clear(1)


def _batched_vs_single_root(g, roots, bopts, popts, torch):
    """Batched levels of every root against the single-root BFS on the
    device; returns the batched levels on the host and the stats."""
    with ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
        dg.sell_build(32, 1024, 1024)
        d = torch.empty((g.n, 64), dtype=torch.int32, device="cuda")
        st = dg.msbfs64_device(roots, d, bopts)
        torch.cuda.synchronize()
        d_lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
        for i, r in enumerate(roots):
            dg.bfs_device(int(r), d_lv, None, popts)
            torch.cuda.synchronize()
            assert torch.equal(d[:, i], d_lv), f"root {r}: batched levels differ"
        cols = [0, 21, 42, 63]
        out = d[:, cols].cpu().numpy()
        single = {}
        for i in cols:
            lv, pa, _ = dg.bfs(int(roots[i]), popts)
            single[i] = (lv, pa)
    return out, cols, single, st


def test_headline_rmat24_64_roots_learned_graph_loop(learned_weights):
    import torch
    g = ab.gen_rmat(24, 16, seed=24)
    roots = g.pick_roots(64, seed=7)
    assert learned_weights.get("batched") and learned_weights.get("plain")
    bopts = ab.bfs_opts("learned", "graph")
    popts = ab.bfs_opts("learned", "graph")
    out, cols, single, st = _batched_vs_single_root(g, roots, bopts, popts, torch)
    # the default budget pushes some small-frontier roots at this scale
    assert st.pushed_roots > 0
    for k, i in enumerate(cols):
        r = int(roots[i])
        olv, opa, _ = oracle.bfs(g.rowptr, g.col, r)
        assert np.array_equal(out[:, k], olv), f"root {r}: batched levels vs oracle"
        lv, pa = single[i]
        assert np.array_equal(lv, olv) and np.array_equal(pa, opa), f"root {r}: single-root"
        assert oracle.validate(g.rowptr, g.col, r, lv, pa) == 0


def test_rmat26_offsets_past_2_31(learned_weights):
    import torch
    g = ab.gen_rmat(26, 17, seed=26)
    assert g.nnz > 2**31
    roots = g.pick_roots(64, seed=7)
    opts = ab.bfs_opts("learned", "graph")
    out, cols, single, _ = _batched_vs_single_root(g, roots, opts, opts, torch)
    r = int(roots[cols[0]])
    olv, opa, _ = oracle.bfs(g.rowptr, g.col, r)
    assert np.array_equal(out[:, 0], olv)
    lv, pa = single[cols[0]]
    assert np.array_equal(lv, olv) and np.array_equal(pa, opa)
    assert oracle.validate(g.rowptr, g.col, r, lv, pa) == 0

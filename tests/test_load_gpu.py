"""GPU parity on graphs loaded from files: the golden Matrix Market inputs
(unsorted rows, repeated entries, self-loops) through alb_graph_read, the
SELL build and both BFS forms, against the oracle."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
RECS = [r for r in json.loads((GOLDEN / "mtx.json").read_text()) if r["name"] != "empty"]


@pytest.mark.parametrize("rec", RECS, ids=lambda r: r["name"])
def test_loaded_graph_bfs_matches_oracle(rec):
    g = ab.read_graph(GOLDEN / rec["file"])
    deg = np.diff(g.rowptr)
    roots = [int(v) for v in np.flatnonzero(deg > 0)[:6]]
    with ab.Graph(g) as dg:
        dg.sell_build()
        for r in roots:
            olv, opa, _ = oracle.bfs(g.rowptr, g.col, r)
            lv, pa, _ = dg.bfs(r, ab.bfs_opts("beamer"))
            assert np.array_equal(lv, olv) and np.array_equal(pa, opa), f"root {r}"
        levels, _ = dg.msbfs64(np.array(roots, np.int32), ab.bfs_opts("beamer"))
        ref = np.stack([oracle.bfs(g.rowptr, g.col, r)[0] for r in roots], 1)
        assert np.array_equal(levels[:, :len(roots)], ref)

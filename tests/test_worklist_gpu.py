"""Persistent work-list BFS and the autotuner: every item's levels equal the
oracle's (and so the single-root path's) bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import albba_gb300 as ab
import oracle
from albba_gb300 import tune

pytestmark = pytest.mark.gpu


def test_worklist_uneven_graphs_bit_exact():
    rng = np.random.default_rng(3)
    wl = ab.Worklist()
    csrs = []
    configs = [(8, 1, 256), (16, 64, 64), (32, 1024, 256), (64, 16384, 0), (32, 1, 8)]
    for i in range(20):
        sc = int(rng.integers(6, 15))
        ef = int(rng.choice([4, 8, 16, 32]))
        g = ab.gen_rmat(sc, ef, seed=100 + i)
        C_, sigma, lr = configs[i % len(configs)]
        dg = ab.Graph(g)
        dg.sell_build(C_, sigma, lr)
        roots = g.pick_roots(min(8, int(np.count_nonzero(g.degrees()))), seed=i)
        wl.add(dg, roots, alpha=float(rng.choice([8, 14, 24])), beta=float(rng.choice([12, 24])))
        csrs.append(g)
    # a grid and a tiny path too (many levels, top-down heavy)
    grid = ab.gen_grid(40, 30, 0.1, 0.002, seed=4)
    dgg = ab.Graph(grid)
    dgg.sell_build(32, 256)
    wl.add(dgg, grid.pick_roots(4, 1))
    csrs.append(grid)
    path = ab.csr_from_edges(100, np.arange(99), np.arange(1, 100))
    dgp = ab.Graph(path)
    dgp.sell_build(16, 1)
    wl.add(dgp, np.array([0, 50, 99], np.int32))
    csrs.append(path)
    for block in (128, 256, 512):
        levels, st = wl.run(block)
        assert st.ms > 0 and st.kernels == 1
        for lv, (gi, root, n) in zip(levels, wl.layout):
            g = csrs[gi]
            ref, _, _ = oracle.bfs(g.rowptr, g.col, root)
            assert np.array_equal(lv, ref), (gi, root, block)


def test_worklist_carries_a_graph_too_large_for_shared_memory():
    """A graph whose three bitmaps exceed one CTA's shared memory (RMAT s20:
    3 x 128 KB) runs its items on the single-root path, into the same output
    and order, beside small graphs that run in the persistent kernel."""
    wl = ab.Worklist()
    csrs = []
    for i, (sc, ef) in enumerate([(10, 8), (20, 8), (12, 16)]):
        g = ab.gen_rmat(sc, ef, seed=300 + i)
        dg = ab.Graph(g)
        dg.sell_build(32, 256)
        wl.add(dg, g.pick_roots(3, seed=i))
        csrs.append(g)
    levels, st = wl.run(256)
    assert st.ms > 0 and st.kernels > 1
    for lv, (gi, root, n) in zip(levels, wl.layout):
        g = csrs[gi]
        ref, _, _ = oracle.bfs(g.rowptr, g.col, root)
        assert np.array_equal(lv, ref), (gi, root)


def test_worklist_rejects_bad_input():
    wl = ab.Worklist()
    g = ab.gen_rmat(8, 8, seed=1)
    dg = ab.Graph(g)
    with pytest.raises(ab.AlbError) as ei:
        wl.add(dg, np.array([0], np.int32))  # no SELL build yet
    assert ei.value.code == ab.ERR_STATE
    dg.sell_build()
    with pytest.raises(ab.AlbError):
        wl.add(dg, np.array([g.n], np.int32))
    with pytest.raises(ab.AlbError):
        ab.Worklist().run()


def test_autotuner_picks_from_grid_and_caches(tmp_path, monkeypatch):
    monkeypatch.setattr(tune, "CACHE", tmp_path / "cache.json")
    g = ab.gen_rmat(12, 16, seed=5)
    roots = g.pick_roots(4, 2)
    grid = {"C": [16, 32], "sigma": [1, 1024], "block": [128, 256], "alpha": [14.0],
            "beta": [24.0], "long_row": [256]}
    p = tune.get(g, roots, grid=grid)
    assert p["C"] in grid["C"] and p["sigma"] in grid["sigma"] and p["block"] in grid["block"]
    assert (tmp_path / "cache.json").exists()
    assert tune.lookup(g) == p
    # same class -> cache hit, no tuning
    g2 = ab.gen_rmat(12, 16, seed=6)
    assert tune.shape_class(g2) == tune.shape_class(g)
    assert tune.get(g2, roots, tune_missing=False) == p
    with tune.build(g, p) as dg:
        for r in roots:
            lv, pa, _ = dg.bfs(int(r), ab.bfs_opts("beamer", "graph", alpha=p["alpha"],
                                                   beta=p["beta"], block=p["block"]))
            olv, opa, _ = oracle.bfs(g.rowptr, g.col, int(r))
            assert np.array_equal(lv, olv) and np.array_equal(pa, opa)

"""GPU parity for the 64-root bit-parallel BFS: every root's levels equal the
oracle's (and therefore the single-root path's) bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import albba_gb300 as ab
import oracle
from conftest import make_graph

pytestmark = pytest.mark.gpu


def oracle_levels(g, roots):
    return np.stack([oracle.bfs(g.rowptr, g.col, int(r))[0] for r in roots], axis=1)


def check(g, dg, roots, opts=None):
    lv, st = dg.msbfs64(roots, opts)
    ref = oracle_levels(g, roots)
    k = len(roots)
    assert np.array_equal(lv[:, :k], ref)
    assert np.all(lv[:, k:] == -1)
    deg = np.diff(g.rowptr)
    assert st.reached == int(np.count_nonzero(ref >= 0))
    assert st.edges == int(sum(deg[ref[:, i] >= 0].sum() for i in range(k)))
    assert st.num_levels == int(ref.max()) + 2 or st.num_levels == int(ref.max()) + 1
    return lv, st


@pytest.fixture(scope="module")
def rmat16_dev(rmat16):
    g, roots = rmat16
    dg = ab.Graph(g)
    dg.sell_build(32, 1024)
    yield g, roots, dg
    dg.close()


@pytest.mark.parametrize("policy", ["beamer", "topdown", "bottomup", "bottomup_nobypass",
                                    "ref004", "learned"])
def test_config0_64_roots(rmat16_dev, policy):
    g, roots, dg = rmat16_dev
    check(g, dg, roots, ab.bfs_opts(policy, "host"))


def test_fewer_roots_and_duplicates(rmat16_dev):
    g, roots, dg = rmat16_dev
    check(g, dg, roots[:5])
    check(g, dg, roots[:1])
    dup = np.array([roots[0], roots[1], roots[0], roots[2]], np.int32)
    check(g, dg, dup)


@pytest.mark.parametrize("spec", [
    {"kind": "grid", "rows": 48, "cols": 40, "drop": 0.1, "shortcut_frac": 0.002, "seed": 14},
    {"kind": "er", "n": 3000, "mean_degree": 4.0, "seed": 15},
    {"kind": "tiny", "name": "path_star"},
], ids=lambda s: s["kind"])
def test_other_families(spec):
    g = make_graph(spec)
    roots = np.arange(min(g.n, 13), dtype=np.int32) if spec["kind"] == "tiny" \
        else g.pick_roots(64, 3)
    with ab.Graph(g) as dg:
        for C_, sigma, long_row in ((32, 1, 256), (16, 256, 4), (64, 64, 0)):
            dg.sell_build(C_, sigma, long_row)
            for policy in ("beamer", "topdown", "bottomup"):
                check(g, dg, roots, ab.bfs_opts(policy))


def test_many_levels_flush_snapshots():
    # a long path: more levels than the snapshot store holds
    n = 300
    u = np.arange(n - 1)
    g = ab.csr_from_edges(n, u, u + 1)
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1)
        lv, st = check(g, dg, np.array([0, 150, 299, 7], np.int32))
        assert st.num_levels > 64
        # the same into page-locked host memory, which the expansion writes
        # directly (its later flushes included)
        import torch
        roots = np.array([0, 150, 299, 7], np.int32)
        pinned = torch.full((n, 64), -7, dtype=torch.int32, pin_memory=True).numpy()
        lv2, _ = dg.msbfs64(roots, out=pinned)
        assert lv2 is pinned and np.array_equal(lv2, lv)


def test_device_output_and_trace(rmat16_dev):
    import torch
    g, roots, dg = rmat16_dev
    d = torch.empty((g.n, 64), dtype=torch.int32, device="cuda")
    st = dg.msbfs64_device(roots, d, ab.bfs_opts("beamer", trace=True))
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), oracle_levels(g, roots))
    tr = dg.level_trace()
    assert len(tr) == st.num_levels
    assert all(t.step_us > 0 for t in tr)
    assert st.levels_topdown + st.levels_bottomup == st.num_levels


def test_bad_roots_rejected(rmat16_dev):
    g, roots, dg = rmat16_dev
    with pytest.raises(ab.AlbError) as ei:
        dg.msbfs64(np.array([g.n], np.int32))
    assert ei.value.code == ab.ERR_INVALID
    with pytest.raises(ab.AlbError):
        dg.msbfs64(np.zeros(65, np.int32))


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_pushed_roots_exact(rmat16_dev, monkeypatch, loop):
    # roots with small frontiers are pushed at the first bottom-up level; a
    # budget of every stored entry (ALB_MS_PUSH_DIV=1) pushes many of them,
    # 0 turns the push off: the levels are the oracle's either way
    g, roots, dg = rmat16_dev
    monkeypatch.setenv("ALB_MS_PUSH_DIV", "1")
    _, st = check(g, dg, roots, ab.bfs_opts("beamer", loop))
    assert st.levels_bottomup > 0
    # popc(tmask) summed over the levels that follow a top-down level
    assert 0 < st.pushed_roots <= len(roots) * st.levels_bottomup
    monkeypatch.setenv("ALB_MS_PUSH_DIV", "0")
    _, st = check(g, dg, roots, ab.bfs_opts("beamer", loop))
    assert st.pushed_roots == 0
    # a smaller root set: only the roots in use are pushed
    monkeypatch.setenv("ALB_MS_PUSH_DIV", "1")
    _, st = check(g, dg, roots[:7], ab.bfs_opts("beamer", loop))
    assert st.pushed_roots <= 7 * st.levels_bottomup


def test_full_scale_against_single_root():
    # RMAT s23: large enough that the pull hands out runs of more than 8
    # words, the pushed roots are chosen from sampled frontiers and the long
    # rows are many; every root's levels equal the single-root BFS (itself
    # oracle-exact at every size tested), and two roots are checked against
    # the oracle directly
    import torch
    g = ab.gen_rmat(23, 16, seed=31)
    roots = g.pick_roots(64, seed=5)
    with ab.Graph(g, flags=ab.CSR_SYMMETRIC | ab.CSR_SORTED) as dg:
        dg.sell_build()
        d = torch.empty((g.n, 64), dtype=torch.int32, device="cuda")
        st = dg.msbfs64_device(roots, d, ab.bfs_opts("beamer"))
        torch.cuda.synchronize()
        assert st.pushed_roots > 0
        d_lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
        for i, r in enumerate(roots):
            dg.bfs_device(int(r), d_lv, None, ab.bfs_opts("beamer"))
            torch.cuda.synchronize()
            assert torch.equal(d[:, i], d_lv), f"root {r}"
        out = d.cpu().numpy()
    for i in (0, 37):
        assert np.array_equal(out[:, i], oracle.bfs(g.rowptr, g.col, int(roots[i]))[0])


def test_host_levels_page_locked_and_pageable(rmat16_dev):
    # page-locked output is written by the expansion across the host link;
    # pageable output goes through a device buffer and a copy: same levels
    import torch
    g, roots, dg = rmat16_dev
    pinned = torch.full((g.n, 64), -7, dtype=torch.int32, pin_memory=True).numpy()
    a, _ = dg.msbfs64(roots, out=pinned)
    b, _ = dg.msbfs64(roots)
    want = oracle_levels(g, roots)
    k = len(roots)
    assert a is pinned
    assert np.array_equal(a[:, :k], want) and np.array_equal(b[:, :k], want)
    assert np.array_equal(a, b)

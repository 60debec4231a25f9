"""GPU parity: single-root BFS levels and parents bit-exact against the oracle,
SELL-C-sigma arrays against the oracle's restatement of the reference builder.
All calls go through the C ABI (libalbba_gb300.so)."""
from __future__ import annotations

import numpy as np
import pytest

import albba_gb300 as ab
import oracle
from conftest import make_graph

pytestmark = pytest.mark.gpu


def transpose(n, rp, col):
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    order = np.lexsort((src, col))
    trp = np.zeros(n + 1, np.int64)
    np.add.at(trp, col.astype(np.int64) + 1, 1)
    return np.cumsum(trp), src[order].astype(np.int32)


def check_root(g, dg, root, opts=None, in_rp=None, in_col=None):
    lv, pa, st = dg.bfs(int(root), opts)
    olv, opa, nl = oracle.bfs(g.rowptr, g.col, int(root), in_rp, in_col)
    assert np.array_equal(lv, olv), f"levels differ at root {root}"
    assert np.array_equal(pa, opa), f"parents differ at root {root}"
    assert st.num_levels == nl
    assert st.reached == int(np.count_nonzero(olv >= 0))
    deg = np.diff(g.rowptr)
    assert st.edges == int(deg[olv >= 0].sum())
    return st


@pytest.fixture(scope="module")
def rmat16_dev(rmat16):
    g, roots = rmat16
    dg = ab.Graph(g)
    dg.sell_build(32, 1024)
    yield g, roots, dg
    dg.close()


def test_config0_all_64_roots_graph_loop(rmat16_dev):
    g, roots, dg = rmat16_dev
    for r in roots:
        check_root(g, dg, r, ab.bfs_opts("beamer", "graph"))


@pytest.mark.parametrize("loop", ["host", "persistent"])
def test_config0_other_loops(rmat16_dev, loop):
    g, roots, dg = rmat16_dev
    for r in roots[:16]:
        check_root(g, dg, r, ab.bfs_opts("beamer", loop))


@pytest.mark.parametrize("policy", ["topdown", "bottomup", "bottomup_nobypass", "ref004"])
@pytest.mark.parametrize("loop", ["graph", "persistent", "host"])
def test_config0_every_policy(rmat16_dev, policy, loop):
    g, roots, dg = rmat16_dev
    for r in roots[:4]:
        check_root(g, dg, r, ab.bfs_opts(policy, loop))


@pytest.mark.parametrize("C_,sigma,long_row", [(32, 1, 256), (32, 1024, 256), (32, 16384, 0),
                                               (8, 64, 64), (16, 256, 1000), (64, 4096, 256),
                                               (64, 1, 0)])
def test_sell_export_matches_oracle(rmat16, C_, sigma, long_row):
    g, roots = rmat16
    with ab.Graph(g) as dg:
        dg.sell_build(C_, sigma, long_row)
        ex = dg.sell_export()
        order = oracle.sell_order(np.diff(g.rowptr).astype(np.int32), sigma)
        inv, width, off, scol = oracle.sell_build(g.rowptr, g.col, order, C_, long_row)
        assert np.array_equal(ex.perm, order)
        assert np.array_equal(ex.width, width)
        assert np.array_equal(ex.slice_off, off)
        assert np.array_equal(ex.col, scol)
        lrow, lptr, lcol = dg.sell_long_export()
        olrow, olptr, olcol = oracle.sell_long(g.rowptr, g.col, order, long_row)
        assert np.array_equal(lrow, olrow) and np.array_equal(lptr, olptr)
        assert np.array_equal(lcol, olcol)
        if long_row > 0:
            assert len(lrow) > 0
        for r in roots[:4]:
            for loop in ("graph", "persistent"):
                check_root(g, dg, r, ab.bfs_opts("beamer", loop))


@pytest.mark.parametrize("spec", [
    {"kind": "grid", "rows": 48, "cols": 40, "drop": 0.1, "shortcut_frac": 0.002, "seed": 14},
    {"kind": "er", "n": 3000, "mean_degree": 4.0, "seed": 15},
    {"kind": "rmat", "scale": 12, "edgefactor": 8, "seed": 12},
    {"kind": "tiny", "name": "path_star"},
], ids=lambda s: s["kind"])
def test_other_families(spec):
    g = make_graph(spec)
    roots = list(range(min(g.n, 13))) if spec["kind"] == "tiny" else g.pick_roots(8, 3).tolist()
    with ab.Graph(g) as dg:
        for C_, sigma, long_row in ((32, 1, 256), (32, 256, 8), (16, 64, 0)):
            dg.sell_build(C_, sigma, long_row)
            for r in roots:
                for loop in ("graph", "host", "persistent"):
                    check_root(g, dg, r, ab.bfs_opts("beamer", loop))
                check_root(g, dg, r, ab.bfs_opts("bottomup_nobypass", "graph"))


def test_isolated_root_and_empty_levels():
    g = make_graph({"kind": "tiny"})
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1)
        st = check_root(g, dg, 10)  # isolated vertex
        assert st.num_levels == 1 and st.reached == 1


def test_directed_graph_both_orientations():
    rng = np.random.default_rng(5)
    n, m = 2000, 9000
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    keep = u != v
    key = np.unique(u[keep].astype(np.int64) * n + v[keep])
    su, sv = (key // n).astype(np.int32), (key % n).astype(np.int32)
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, su.astype(np.int64) + 1, 1)
    rp = np.cumsum(rp)
    out_csr = ab.Csr(rp, sv)
    in_rp, in_col = transpose(n, rp, sv)
    roots = [0, 17, 512, 1999]
    dg = ab.Graph(out_csr, flags=ab.CSR_OUT)
    dg.sell_build(32, 256)
    dg2 = ab.Graph(ab.Csr(in_rp, in_col), flags=ab.CSR_IN)
    dg2.sell_build(32, 256)
    for r in roots:
        olv, opa, nl = oracle.bfs(rp, sv, r, in_rp, in_col)
        for d in (dg, dg2):
            for loop in ("graph", "persistent"):
                lv, pa, st = d.bfs(r, ab.bfs_opts("beamer", loop))
                assert np.array_equal(lv, olv) and np.array_equal(pa, opa)
        assert oracle.validate(rp, sv, r, olv, opa, in_rp, in_col) == 0
    dg.close()
    dg2.close()


def test_unsorted_rows_are_sorted_on_upload():
    g = make_graph({"kind": "rmat", "scale": 11, "edgefactor": 16, "seed": 3})
    col = g.col.copy()
    rng = np.random.default_rng(1)
    for v in range(g.n):
        a, b = g.rowptr[v], g.rowptr[v + 1]
        rng.shuffle(col[a:b])
    with ab.Graph(ab.Csr(g.rowptr, col)) as dg:
        dg.sell_build(32, 1024)
        for r in g.pick_roots(4, 1):
            check_root(g, dg, r)


def test_int32_graph_entry_point():
    g = make_graph({"kind": "rmat", "scale": 11, "edgefactor": 16, "seed": 3})
    dg = ab.Graph.from_int32(g.n, g.rowptr.astype(np.int32), g.col, ab.CSR_SYMMETRIC)
    dg.sell_build()
    for r in g.pick_roots(4, 2):
        check_root(g, dg, r)
    dg.close()


def test_trace_records_levels(rmat16_dev):
    g, roots, dg = rmat16_dev
    for loop in ("graph", "host", "persistent"):
        lv, pa, st = dg.bfs(int(roots[0]), ab.bfs_opts("beamer", loop, trace=True))
        tr = dg.level_trace()
        assert len(tr) == st.num_levels
        counts = np.bincount(lv[lv >= 0])
        assert [t.nf for t in tr] == counts.tolist()
        assert [t.level for t in tr] == list(range(st.num_levels))
        assert sum(t.dir == ab.DIR_TOPDOWN for t in tr) == st.levels_topdown
        assert tr[0].dir == ab.DIR_TOPDOWN


def test_device_outputs(rmat16_dev):
    import torch
    g, roots, dg = rmat16_dev
    d_lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
    d_pa = torch.empty(g.n, dtype=torch.int32, device="cuda")
    st = dg.bfs_device(int(roots[1]), d_lv, d_pa)
    torch.cuda.synchronize()
    olv, opa, nl = oracle.bfs(g.rowptr, g.col, int(roots[1]))
    assert np.array_equal(d_lv.cpu().numpy(), olv)
    assert np.array_equal(d_pa.cpu().numpy(), opa)
    assert st.ms > 0


def test_errors_are_status_codes(rmat16):
    g, roots = rmat16
    with ab.Graph(g) as dg:
        with pytest.raises(ab.AlbError) as ei:
            dg.bfs(0)
        assert ei.value.code == ab.ERR_STATE
        dg.sell_build()
        with pytest.raises(ab.AlbError) as ei:
            dg.bfs(g.n)
        assert ei.value.code == ab.ERR_INVALID
        with pytest.raises(ab.AlbError) as ei:
            dg.sell_build(12, 64)
        assert ei.value.code == ab.ERR_UNSUPPORTED
        with pytest.raises(ab.AlbError) as ei:
            dg.sell_build(32, 20000)
        assert ei.value.code == ab.ERR_UNSUPPORTED
        # the graph stays usable after rejected calls
        dg.sell_build()
        check_root(g, dg, roots[0])


def test_injected_allocation_failure_is_clean(rmat16):
    g, roots = rmat16
    for k in (1, 2, 5, 12):
        ab.debug_fail_alloc_after(k)
        try:
            dg = ab.Graph(g)
            dg.sell_build()
            dg.bfs(int(roots[0]))
            dg.close()
        except ab.AlbError as e:
            assert e.code == ab.ERR_OOM and "injected" in ab.last_error()
        finally:
            ab.debug_fail_alloc_after(0)
    with ab.Graph(g) as dg:
        dg.sell_build()
        check_root(g, dg, roots[0])


def test_scale20_levels_and_validation():
    g = ab.gen_rmat(20, 16, seed=2020)
    roots = g.pick_roots(4, 11)
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1024)
        for r in roots:
            for loop in ("graph", "persistent"):
                lv, pa, st = dg.bfs(int(r), ab.bfs_opts("beamer", loop))
                olv, opa, nl = oracle.bfs(g.rowptr, g.col, int(r))
                assert np.array_equal(lv, olv) and np.array_equal(pa, opa)
            assert oracle.validate(g.rowptr, g.col, int(r), lv, pa) == 0


@pytest.mark.parametrize("scale,staged", [(18, True), (21, False)])
def test_frontier_staged_and_global_slice_passes(scale, staged):
    """The bottom-up slice pass stages the frontier bitmap in shared memory
    while it fits (192 KB: n up to 1.5M rows) and gathers from global memory
    beyond; both kernels, on every policy that pulls, match the oracle."""
    g = ab.gen_rmat(scale, 8, seed=1800 + scale)
    assert (g.n <= 192 * 1024 * 8) == staged
    roots = g.pick_roots(2, 3)
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1024)
        for r in roots:
            olv, opa, _ = oracle.bfs(g.rowptr, g.col, int(r))
            for policy in ("bottomup", "bottomup_nobypass", "beamer"):
                for loop in ("graph", "host"):
                    lv, pa, _ = dg.bfs(int(r), ab.bfs_opts(policy, loop))
                    assert np.array_equal(lv, olv) and np.array_equal(pa, opa), (policy, loop)


@pytest.mark.parametrize("policy", ["beamer", "topdown", "bottomup", "ref004"])
def test_persistent_lazy_levels_on_a_grid(policy):
    """The persistent loop runs small top-down levels lazily (one grid
    barrier per level, targets claimed on their level word, the bitmaps left
    stale) and rebuilds the visited and frontier bitmaps when a level that
    reads them follows (a large top-down level or a bottom-up one). A grid
    with shortcuts has long runs of small levels and frontiers that grow past
    the lazy limit: every switch is taken, and the levels, parents and
    per-level counters match the oracle and the other loop drivers."""
    g = ab.gen_grid(300, 300, 0.1, 2e-4, seed=21)
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1)
        for r in g.pick_roots(4, seed=5):
            olv, opa, nl = oracle.bfs(g.rowptr, g.col, int(r))
            lv, pa, st = dg.bfs(int(r), ab.bfs_opts(policy, "persistent", trace=True))
            assert np.array_equal(lv, olv) and np.array_equal(pa, opa), (policy, int(r))
            assert st.num_levels == nl
            pers = [(t.dir, t.nf, t.mf, t.nu, t.mu, t.bytes) for t in dg.level_trace()]
            lv2, pa2, _ = dg.bfs(int(r), ab.bfs_opts(policy, "host", trace=True))
            host = [(t.dir, t.nf, t.mf, t.nu, t.mu, t.bytes) for t in dg.level_trace()]
            assert pers == host

"""Device-side graph ingest: the CSR checks, the row sort, the transpose with
ascending rows (the reference's counting transpose, bfs/src/sparse_matrix.c:
230-290), the symmetry test and the reference driver's undirected merge
(bfs/src/main.c:127-163, MergeArr at bfs/src/utils.c:351-379), all run on
the GPU by alb_graph_create / alb_graph_create_undirected / alb_graph_load.
Integer outputs: compared exactly."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def rows_of(rp):
    return np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp))


def sorted_csr(n, rows, cols):
    """CSR with rows ascending (stable): numpy's restatement of a counting sort."""
    order = np.lexsort((cols, rows))
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, np.asarray(rows, np.int64) + 1, 1)
    return np.cumsum(rp), np.asarray(cols, np.int32)[order]


def directed(n, m, seed, hubs=()):
    """Random directed edges with duplicates and self-loops kept, plus hub
    targets with the given in-degrees (rows of every sort class)."""
    rng = np.random.default_rng(seed)
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    for h, deg in hubs:
        u = np.concatenate([u, rng.integers(0, n, deg)])
        v = np.concatenate([v, np.full(deg, h)])
    return u.astype(np.int64), v.astype(np.int32)


def shuffled_rows(rp, col, seed):
    """The same CSR with every row's entries in random order."""
    rng = np.random.default_rng(seed)
    rows = rows_of(rp)
    key = rng.random(col.shape[0])
    order = np.lexsort((key, rows))
    return rp, col[order]


def test_bad_inputs_refused_on_the_device():
    h = C.c_void_p()
    lib = ab.lib()
    cases = [
        (np.array([0, 1, 2], np.int64), np.array([0, 5], np.int32)),    # column >= n
        (np.array([0, 1, 2], np.int64), np.array([0, -1], np.int32)),   # negative column
        (np.array([0, 2, 1, 2], np.int64), np.array([1, 0], np.int32)),  # offsets decrease
    ]
    for rp, col in cases:
        n = len(rp) - 1
        for flags in (ab.CSR_SYMMETRIC, ab.CSR_IN, ab.CSR_OUT):
            code = lib.alb_graph_create(n, rp.ctypes.data, col.ctypes.data, flags, C.byref(h))
            assert code == ab.ERR_INVALID and not h.value, (rp, col, flags)
        code = lib.alb_graph_create_undirected(n, rp.ctypes.data, col.ctypes.data, C.byref(h))
        assert code == ab.ERR_INVALID and not h.value
    # the device stays usable
    g = ab.gen_rmat(10, 8, seed=1)
    with ab.Graph(g) as dg:
        dg.sell_build()
        lv, pa, _ = dg.bfs(0)
        olv, opa, _ = oracle.bfs(g.rowptr, g.col, 0)
        assert np.array_equal(lv, olv) and np.array_equal(pa, opa)


def test_unsorted_rows_are_sorted_on_the_device():
    g = ab.gen_rmat(16, 16, seed=2024)  # rows up to thousands of entries
    rp, col = shuffled_rows(g.rowptr, g.col, seed=3)
    assert not np.array_equal(col, g.col)
    with ab.Graph(ab.Csr(rp, col), flags=ab.CSR_SYMMETRIC) as dg:
        back = dg.export_csr(0)
        assert np.array_equal(back.rowptr, g.rowptr) and np.array_equal(back.col, g.col)
        dg.sell_build()
        for r in g.pick_roots(3, seed=7):
            lv, pa, _ = dg.bfs(int(r))
            olv, opa, _ = oracle.bfs(g.rowptr, g.col, int(r))
            assert np.array_equal(lv, olv) and np.array_equal(pa, opa)


@pytest.mark.parametrize("flags", [ab.CSR_OUT, ab.CSR_IN])
def test_directed_transpose_on_the_device(flags):
    n = 1 << 15
    # in-degrees of every row-sort class: <= 32, <= 4096 and two long rows
    u, v = directed(n, 200_000, seed=9, hubs=((7, 3000), (11, 9000), (12345, 70000)))
    rp, col = sorted_csr(n, u, v)             # row u: targets, ascending
    trp, tcol = sorted_csr(n, v, u)           # its transpose, rows ascending
    srp, scol = shuffled_rows(rp, col, seed=4)
    with ab.Graph(ab.Csr(srp, scol), flags=flags) as dg:
        assert not dg.symmetric
        given, other = (1, 0) if flags == ab.CSR_OUT else (0, 1)
        a = dg.export_csr(given)
        b = dg.export_csr(other)
        assert np.array_equal(a.rowptr, rp) and np.array_equal(a.col, col)
        assert np.array_equal(b.rowptr, trp) and np.array_equal(b.col, tcol)
        if flags == ab.CSR_OUT:  # BFS along the edges: the oracle's directed form
            dg.sell_build()
            for root in (0, 7, 999):
                lv, pa, _ = dg.bfs(root)
                olv, opa, _ = oracle.bfs(rp, col, root, trp, tcol)
                assert np.array_equal(lv, olv) and np.array_equal(pa, opa)


def test_symmetric_input_is_detected():
    g = ab.gen_rmat(14, 16, seed=5)
    for flags in (ab.CSR_IN, ab.CSR_OUT):
        with ab.Graph(g, flags=flags) as dg:
            assert dg.symmetric
            a, b = dg.export_csr(0), dg.export_csr(1)
            assert np.array_equal(a.col, g.col) and np.array_equal(b.col, g.col)
    # the reference's int32 CSR as the plugin passes it (its working matrix)
    rp32 = g.rowptr.astype(np.int32)
    with ab.Graph.from_int32(g.n, rp32, g.col, ab.CSR_IN) as dg:
        assert dg.symmetric


def _golden_rows_sorted(rowptr, col):
    rp = np.asarray(rowptr, np.int64)
    c = np.asarray(col, np.int32)
    return sorted_csr(len(rp) - 1, rows_of(rp), c)


RECS = json.loads((GOLDEN / "mtx.json").read_text())


@pytest.mark.parametrize("rec", [r for r in RECS if not r["symmetric"]], ids=lambda r: r["name"])
def test_undirected_merge_on_the_device_matches_reference(rec):
    # the golden records hold the reference driver's own merge; the device
    # graph keeps the same entries with every row sorted
    g, _ = ab.read_mtx(GOLDEN / rec["file"])
    want_rp, want_col = _golden_rows_sorted(rec["undirected_rowptr"], rec["undirected_col"])
    with ab.Graph.undirected(g) as dg:
        assert dg.symmetric
        got = dg.export_csr(0)
    assert np.array_equal(got.rowptr, want_rp) and np.array_equal(got.col, want_col)


@pytest.mark.parametrize("rec", RECS, ids=lambda r: r["name"])
def test_graph_load_onto_the_device(rec):
    key = "rowptr" if rec["symmetric"] else "undirected_rowptr"
    ckey = "col" if rec["symmetric"] else "undirected_col"
    want_rp, want_col = _golden_rows_sorted(rec[key], rec[ckey])
    with ab.Graph.load(GOLDEN / rec["file"]) as dg:
        got = dg.export_csr(0)
    assert np.array_equal(got.rowptr, want_rp) and np.array_equal(got.col, want_col)


def test_undirected_merge_at_scale_matches_host_restatement():
    # unsorted rows, duplicates and hubs: the host restatement of the
    # reference's merge (pinned to the golden records) against the device one
    n = 1 << 16
    u, v = directed(n, 600_000, seed=12, hubs=((3, 20000),))
    rp, col = sorted_csr(n, u, v)
    srp, scol = shuffled_rows(rp, col, seed=6)
    host = ab.csr_undirected(ab.Csr(srp, scol))
    want_rp, want_col = sorted_csr(n, rows_of(host.rowptr), host.col)
    with ab.Graph.undirected(ab.Csr(srp, scol)) as dg:
        got = dg.export_csr(0)
        assert np.array_equal(got.rowptr, want_rp) and np.array_equal(got.col, want_col)
        dg.sell_build()
        lv, pa, _ = dg.bfs(3)
    olv, opa, _ = oracle.bfs(want_rp, want_col, 3)
    assert np.array_equal(lv, olv) and np.array_equal(pa, opa)


def _visited_bits(n, visited):
    bits = np.zeros((n + 31) // 32, np.uint32)
    ids = np.flatnonzero(visited)
    np.bitwise_or.at(bits, ids >> 5, (np.uint32(1) << (ids & 31).astype(np.uint32)))
    return bits


@pytest.mark.parametrize("directed_graph", [False, True])
def test_spmspv_merge_is_the_sorted_unvisited_union(directed_graph):
    """alb_spmspv_merge against the reference's push-merge semantics
    (csc_spmspv_merge, bfs/src/bfs_par_kernels.c:350-416, and the task merge
    of bfs/src/bfs_SELLCSv2.c:530-575): the ascending, duplicate-free list of
    the frontier's out-neighbours that are not visited."""
    rng = np.random.default_rng(3)
    if directed_graph:
        n = 1 << 14
        u, v = directed(n, 120_000, seed=8, hubs=((5, 6000),))
        rp, col = sorted_csr(n, u, v)
        dg = ab.Graph(ab.Csr(rp, col), flags=ab.CSR_OUT)
    else:
        g = ab.gen_rmat(16, 16, seed=2024)
        n, rp, col = g.n, g.rowptr, g.col
        dg = ab.Graph(g)
    with dg:
        for nx, pv in ((1, 0.0), (37, 0.3), (2000, 0.5), (n // 2, 0.1), (0, 0.0)):
            x = rng.choice(n, nx, replace=False).astype(np.int32)
            visited = rng.random(n) < pv
            got = dg.spmspv_merge(x, _visited_bits(n, visited))
            nbrs = np.concatenate([col[rp[u]:rp[u + 1]] for u in x]) if nx else np.zeros(0, np.int32)
            want = np.unique(nbrs)
            want = want[~visited[want]]
            assert np.array_equal(got, want), nx
        with pytest.raises(ab.AlbError) as ei:
            dg.spmspv_merge(np.array([n], np.int32), _visited_bits(n, np.zeros(n, bool)))
        assert ei.value.code == ab.ERR_INVALID


@pytest.mark.parametrize("at", [1, 2, 3, 4, 5, 127, 128, 1023, -1])
def test_one_descent_inside_one_row_is_found(at):
    """Rows sorted everywhere but one descent inside a row, at entry `at` of
    the column array (every offset of a 16-byte group, the last entry, or the
    next entry when `at` starts a row); around it, empty rows and rows
    starting below their predecessor's last entry (descents at row starts,
    which are allowed). The graph must come back with every row sorted."""
    rng = np.random.default_rng(at + 10)
    n = 600
    lens = rng.integers(0, 8, n)
    lens[::7] = 0
    lens[-1] = 5
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(lens)
    nnz = int(rp[-1])
    assert nnz > 1024
    col = np.empty(nnz, np.int32)
    for r in range(n):
        col[rp[r]:rp[r + 1]] = np.sort(rng.choice(n, rp[r + 1] - rp[r], replace=False))
    e = at % nnz
    while e in set(rp.tolist()):  # a row start: take the next entry
        e += 1
    col[e - 1], col[e] = col[e], col[e - 1]
    starts = set(rp[:-1][rp[:-1] < rp[1:]].tolist())
    inner = [int(d) for d in np.nonzero(col[1:] < col[:-1])[0] + 1 if int(d) not in starts]
    assert inner == [e]
    with ab.Graph(ab.Csr(rp, col), flags=ab.CSR_IN) as dg:
        back = dg.export_csr(0)  # the given side
    want = col.copy()
    for q in range(n):
        want[rp[q]:rp[q + 1]] = np.sort(want[rp[q]:rp[q + 1]])
    assert np.array_equal(back.rowptr, rp) and np.array_equal(back.col, want)

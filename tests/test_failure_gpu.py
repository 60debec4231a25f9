"""Failure detection on the device, without a GPU fault: every device-side
wait (the persistent loop's grid barrier, the no-alloc BFS's grid barrier,
the staged pull's bulk-copy wait) is bounded and reports ALB_ERR_TIMEOUT.
A test hook shortens the bound to milliseconds and makes the wait run out --
a block skips its barrier arrival, or the bulk-copy barrier expects bytes
that never come -- and the test checks the status and that the next call on
the same graph is correct. (The reference has no failure handling: it exits
the process, bfs/src/utils.c:102-109.)"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture
def hooks():
    yield ab.debug_device_waits
    ab.debug_device_waits()


@pytest.fixture(scope="module")
def graph(rmat16):
    g, roots = rmat16
    dg = ab.Graph(g)
    dg.sell_build()
    yield g, roots, dg
    dg.close()


def _check(g, dg, root, loop):
    lv, pa, _ = dg.bfs(int(root), ab.bfs_opts("beamer", loop))
    olv, opa, _ = oracle.bfs(g.rowptr, g.col, int(root))
    assert np.array_equal(lv, olv) and np.array_equal(pa, opa)


@pytest.mark.parametrize("level,block", [(0, 0), (1, 5), (2, 151)])
def test_persistent_barrier_timeout_then_recovery(graph, hooks, level, block):
    g, roots, dg = graph
    r = int(roots[0])
    hooks(withhold_level=level, withhold_block=block, timeout_us=2000)
    with pytest.raises(ab.AlbError) as ei:
        dg.bfs(r, ab.bfs_opts("beamer", "persistent"))
    assert ei.value.code == ab.ERR_TIMEOUT
    hooks()
    for loop in ("persistent", "graph"):
        _check(g, dg, r, loop)


def test_bulk_copy_wait_timeout_then_recovery(graph, hooks):
    g, roots, dg = graph
    assert g.n <= 192 * 1024 * 8  # the staged (bulk-copy) pull is used
    r = int(roots[1])
    hooks(short_bulk=True, timeout_us=1000)
    for loop in ("host", "graph"):
        with pytest.raises(ab.AlbError) as ei:
            dg.bfs(r, ab.bfs_opts("bottomup", loop))
        assert ei.value.code == ab.ERR_TIMEOUT
    hooks()
    for loop in ("host", "graph"):
        lv, pa, _ = dg.bfs(r, ab.bfs_opts("bottomup", loop))
        olv, opa, _ = oracle.bfs(g.rowptr, g.col, r)
        assert np.array_equal(lv, olv) and np.array_equal(pa, opa)


def test_noalloc_barrier_timeout_then_recovery(rmat16, hooks):
    import torch
    g, roots = rmat16
    f = ab.lib().alb_bfs_csr_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                  C.c_void_p, C.c_void_p]
    rp = torch.from_numpy(g.rowptr).cuda()
    col = torch.from_numpy(g.col).cuda()
    lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
    pa = torch.empty(g.n, dtype=torch.int32, device="cuda")
    r = int(roots[2])
    hooks(withhold_level=1, withhold_block=3, timeout_us=2000)
    code = f(g.n, rp.data_ptr(), col.data_ptr(), 1, r, lv.data_ptr(), pa.data_ptr(), None)
    assert code == ab.ERR_TIMEOUT
    hooks()
    code = f(g.n, rp.data_ptr(), col.data_ptr(), 1, r, lv.data_ptr(), pa.data_ptr(), None)
    assert code == ab.OK, ab.last_error()
    olv, opa, _ = oracle.bfs(g.rowptr, g.col, r)
    assert np.array_equal(lv.cpu().numpy(), olv) and np.array_equal(pa.cpu().numpy(), opa)

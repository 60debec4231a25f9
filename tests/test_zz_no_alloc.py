"""alb_bfs_csr_noalloc: the BFS entry point for callers that cannot call
cudaMalloc (for example a plug-in whose process's device memory belongs to
another allocator). Called through the C ABI with device buffers the test
owns; its levels and parents must equal those of the allocating entry point
alb_bfs and of the oracle (the CPU restatement of the reference verifier)
exactly (integer outputs: zero tolerance), on two calls in a row (the second
call reuses the library's fixed scratch array and must not see the first
call's contents), up to the largest graph its scratch holds (2^20 vertices).
Collected last so that a failure here cannot stop the other tests of a
run."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

pytestmark = pytest.mark.gpu


def _fn():
    f = ab.lib().alb_bfs_csr_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                  C.c_void_p, C.c_void_p]
    return f


def _reference(csr, root, flags):
    with ab.Graph(csr, flags=flags) as dg:
        dg.sell_build(32, 1024)
        lv, pa, _ = dg.bfs(int(root))
    return lv, pa


def _noalloc(csr, root, symmetric):
    import torch
    rp = torch.from_numpy(np.ascontiguousarray(csr.rowptr, np.int64)).cuda()
    col = torch.from_numpy(np.ascontiguousarray(csr.col, np.int32)).cuda()
    lv = torch.full((csr.n,), 7, dtype=torch.int32, device="cuda")
    pa = torch.full((csr.n,), 7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    code = _fn()(csr.n, rp.data_ptr(), col.data_ptr(), 1 if symmetric else 0, int(root),
                 lv.data_ptr(), pa.data_ptr(), None)
    assert code == ab.OK, ab.last_error()
    torch.cuda.synchronize()
    return lv.cpu().numpy(), pa.cpu().numpy()


def _directed(n, m, seed):
    """Random directed graph: out-CSR and the in-CSR (its transpose)."""
    rng = np.random.default_rng(seed)
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    keep = u != v
    key = np.unique(u[keep].astype(np.int64) * n + v[keep])
    su, sv = (key // n).astype(np.int32), (key % n).astype(np.int32)

    def csr(rows, cols):
        order = np.lexsort((cols, rows))
        rp = np.zeros(n + 1, np.int64)
        np.add.at(rp, rows.astype(np.int64) + 1, 1)
        return ab.Csr(np.cumsum(rp), cols[order].astype(np.int32))

    return csr(su, sv), csr(sv, su)


@pytest.mark.parametrize("scale", [16, 20])
def test_noalloc_matches_alb_bfs_on_two_calls_in_a_row(scale):
    # scale 20 is n = 2^20, the largest graph the fixed scratch holds
    g = ab.gen_rmat(scale, 16, seed=2024)
    assert g.n <= 1 << 20
    roots = g.pick_roots(2, seed=7)
    for root in roots:  # two calls in a row, different roots
        want_lv, want_pa = _reference(g, root, ab.CSR_SYMMETRIC)
        olv, opa, _ = oracle.bfs(g.rowptr, g.col, int(root))
        lv, pa = _noalloc(g, root, symmetric=True)
        assert np.array_equal(lv, want_lv) and np.array_equal(lv, olv)
        assert np.array_equal(pa, want_pa) and np.array_equal(pa, opa)


@pytest.mark.parametrize("n,m", [(5000, 30000), (1 << 20, 6 << 20)])
def test_noalloc_directed_top_down_matches_alb_bfs(n, m):
    out, inn = _directed(n, m, seed=5)
    for root in (0, 1234):  # two calls in a row
        want_lv, want_pa = _reference(out, root, ab.CSR_OUT)
        olv, opa, _ = oracle.bfs(out.rowptr, out.col, root, inn.rowptr, inn.col)
        lv, pa = _noalloc(out, root, symmetric=False)
        assert np.array_equal(lv, want_lv) and np.array_equal(lv, olv)
        assert np.array_equal(pa, want_pa) and np.array_equal(pa, opa)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    n = (1 << 20) + 1
    rp = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    col = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.zeros(1, dtype=torch.int32, device="cuda")
    code = _fn()(n, rp.data_ptr(), col.data_ptr(), 1, 0, out.data_ptr(), out.data_ptr(), None)
    assert code == ab.ERR_UNSUPPORTED and "scratch" in ab.last_error()

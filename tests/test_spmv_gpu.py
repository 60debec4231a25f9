"""fp64 SELL-C-sigma SpMV on the GPU (alb_sellmat_*): y bit-identical to the
reference's kernel_SELLCS_DFC (bfs/src/bfs_par_kernels.c:8-53) -- through
its golden records -- and to the oracle on larger matrices. Floating point,
but the operations and their order are the reference's, so the tolerance is
zero: every bit of y must match."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

GOLDEN_DIR = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN_DIR))
from spmv_cases import CASES, GOLDEN, digest, inputs  # noqa: E402

pytestmark = pytest.mark.gpu
RECS = json.loads(GOLDEN.read_text())


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
@pytest.mark.parametrize("sigma", [1, 256, 16384])
def test_gpu_spmv_matches_reference_bits(case, sigma):
    n, rp, col, val, x = inputs(case)
    with ab.SellMatrix(rp, col, val, sigma) as m:
        assert m.nnz == int(rp[-1]) and m.stored >= m.nnz
        y = m.spmv(x)
        y2 = m.spmv(x)  # a second call on the same matrix
    rec = next(r for r in RECS if r["case"] == case["name"])
    assert [f"{v:016x}" for v in y[:16].view(np.uint64)] == rec["head_bits"]
    assert digest(y) == rec["sha256"]
    assert np.array_equal(y.view(np.uint64), y2.view(np.uint64))


@pytest.mark.parametrize("scale", [18, 22])
def test_gpu_spmv_large_against_oracle(scale):
    import torch
    g = ab.gen_rmat(scale, 16, seed=40 + scale)
    rng = np.random.default_rng(scale)
    val = rng.uniform(-1.0, 1.0, g.nnz) * np.exp2(rng.integers(-20, 20, g.nnz))
    x = rng.standard_normal(g.n)
    want = oracle.spmv(g.rowptr, g.col, val, x)
    with ab.SellMatrix(g.rowptr, g.col, val, 1024) as m:
        dx = torch.from_numpy(x).cuda()
        dy = torch.full((g.n,), float("nan"), dtype=torch.float64, device="cuda")
        us = m.spmv_device(dx, dy)
        assert us > 0
        got = dy.cpu().numpy()
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_gpu_spmv_rejects_bad_input():
    rp = np.array([0, 1, 2], np.int64)
    with pytest.raises(ab.AlbError) as ei:
        ab.SellMatrix(rp, np.array([0, 7], np.int32), np.ones(2))
    assert ei.value.code == ab.ERR_INVALID
    with pytest.raises(ab.AlbError) as ei:
        ab.SellMatrix(rp, np.array([0, 1], np.int32), np.ones(2), sigma=0)
    assert ei.value.code == ab.ERR_UNSUPPORTED


def test_gpu_spmv_long_rows_keep_csr_order():
    """Rows at and past the warp-per-row threshold (511, 512, 513, 1000 and a
    40000-entry hub with repeated columns, so that order matters) next to
    short rows: every y bit equals the oracle's in-order chain."""
    rng = np.random.default_rng(7)
    n = 4096
    lens = rng.integers(0, 24, n)
    lens[[3, 100, 101, 2000, 4095]] = [511, 512, 513, 1000, 40000]
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(lens)
    col = rng.integers(0, n, int(rp[-1])).astype(np.int32)
    col[rp[4095]:rp[4095] + 64] = 17  # one column repeated inside the hub
    val = rng.uniform(-1.0, 1.0, int(rp[-1])) * np.exp2(rng.integers(-30, 30, int(rp[-1])))
    x = rng.standard_normal(n) * np.exp2(rng.integers(-10, 10, n))
    want = oracle.spmv(rp, col, val, x)
    for sigma in (1, 4096):
        with ab.SellMatrix(rp, col, val, sigma) as m:
            got = m.spmv(x)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), sigma

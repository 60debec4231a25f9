"""The oracle's fp64 SpMV against the reference's own (golden records of
tests/golden/make_golden_spmv.py: convert_csr_to_sellcs_dfc +
kernel_SELLCS_DFC, bfs/src/sparse_matrix.c:523-623 and
bfs/src/bfs_par_kernels.c:8-53), bit for bit. CPU only."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLDEN_DIR = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN_DIR))
from spmv_cases import CASES, GOLDEN, digest, inputs  # noqa: E402

RECS = json.loads(GOLDEN.read_text())


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_oracle_spmv_matches_reference_bits(case):
    n, rp, col, val, x = inputs(case)
    y = oracle.spmv(rp, col, val, x)
    recs = [r for r in RECS if r["case"] == case["name"]]
    assert recs
    for r in recs:  # the reference's result does not depend on sigma
        assert r["n"] == n and r["nnz"] == int(rp[-1])
        assert [f"{v:016x}" for v in y[:16].view(np.uint64)] == r["head_bits"]
        assert digest(y) == r["sha256"]


def test_order_of_operations_matters_here():
    # the "wide" case spreads magnitudes over 60 binades, so a different
    # summation order (plain sum of products) changes some bits: the golden
    # records pin the fused, CSR-ordered chain and not just the values
    case = next(c for c in CASES if c["values"] == "wide")
    n, rp, col, val, x = inputs(case)
    y = oracle.spmv(rp, col, val, x)
    rows = np.repeat(np.arange(n), np.diff(rp))
    alt = np.zeros(n)
    np.add.at(alt, rows[::-1], (val * x[col])[::-1])
    assert not np.array_equal(alt.view(np.uint64), y.view(np.uint64))

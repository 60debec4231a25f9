"""Seeded inputs of the fp64 SELL-C-sigma SpMV golden records: the matrices
(generated graphs, and a non-symmetric matrix with duplicate entries, empty
rows, diagonal entries and rows in random order), their values and x.
Shared by make_golden_spmv.py (which runs the reference's own code on them)
and the tests (which run the oracle and the GPU on them)."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

CASES = [
    {"name": "rmat10_ones", "graph": {"kind": "rmat", "scale": 10, "edgefactor": 16, "seed": 11},
     "values": "ones", "x_seed": 1},
    {"name": "rmat12_uniform", "graph": {"kind": "rmat", "scale": 12, "edgefactor": 8, "seed": 12},
     "values": "uniform", "value_seed": 2, "x_seed": 3},
    {"name": "er3000_uniform", "graph": {"kind": "er", "n": 3000, "mean_degree": 4.0, "seed": 15},
     "values": "uniform", "value_seed": 4, "x_seed": 5},
    {"name": "random_dups_diag", "graph": {"kind": "random", "n": 1500, "m": 20000, "seed": 21},
     "values": "wide", "value_seed": 6, "x_seed": 7},
]


def matrix(spec: dict):
    """(n, rowptr int64, col int32) of a case's matrix."""
    import albba_gb300 as ab
    k = spec["kind"]
    if k == "rmat":
        g = ab.gen_rmat(spec["scale"], spec["edgefactor"], spec["seed"])
    elif k == "er":
        g = ab.gen_er(spec["n"], spec["mean_degree"], spec["seed"])
    else:
        rng = np.random.default_rng(spec["seed"])
        n, m = spec["n"], spec["m"]
        rows = rng.integers(0, n - 50, m)  # the last 50 rows stay empty
        cols = rng.integers(0, n, m)
        rows = np.concatenate([rows, np.arange(0, n - 50, 3)])  # diagonal entries
        cols = np.concatenate([cols, np.arange(0, n - 50, 3)])
        dup = rng.integers(0, rows.shape[0], 2000)  # repeated entries
        rows = np.concatenate([rows, rows[dup]])
        cols = np.concatenate([cols, cols[dup]])
        order = np.lexsort((rng.random(rows.shape[0]), rows))  # rows in random order inside
        rp = np.zeros(n + 1, np.int64)
        np.add.at(rp, rows + 1, 1)
        return n, np.cumsum(rp), cols[order].astype(np.int32)
    return g.n, g.rowptr.astype(np.int64), g.col.astype(np.int32)


def inputs(case: dict):
    """(n, rowptr, col, values float64, x float64) of a case."""
    n, rp, col = matrix(case["graph"])
    nnz = int(rp[-1])
    if case["values"] == "ones":
        val = np.ones(nnz)
    elif case["values"] == "uniform":
        val = np.random.default_rng(case["value_seed"]).uniform(-1.0, 1.0, nnz)
    else:  # magnitudes over many binades, so that rounding order shows
        rng = np.random.default_rng(case["value_seed"])
        val = rng.uniform(-1.0, 1.0, nnz) * np.exp2(rng.integers(-30, 30, nnz))
    x = np.random.default_rng(case["x_seed"]).standard_normal(n)
    return n, rp, col, val, x


def digest(y: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(y, np.float64).tobytes()).hexdigest()


GOLDEN = Path(__file__).resolve().parent / "spmv.json"

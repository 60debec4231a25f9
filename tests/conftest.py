"""Shared test setup: marker registration, in-tree builds, small helpers."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # make sure the native library and the oracle exist before collection
    import __graft_entry__ as ge  # noqa: WPS433
    _b = ge._build_module()
    if not _b.LIB.exists():
        _b.build_library()
    import oracle  # noqa: WPS433
    if not oracle.LIB.exists():
        oracle.build()


def load_golden(name: str):
    return json.loads((GOLDEN / name).read_text())


def make_graph(spec: dict):
    import albba_gb300 as ab
    k = spec["kind"]
    if k == "rmat":
        return ab.gen_rmat(spec["scale"], spec["edgefactor"], spec["seed"])
    if k == "grid":
        return ab.gen_grid(spec["rows"], spec["cols"], spec["drop"], spec["shortcut_frac"],
                           spec["seed"])
    if k == "er":
        return ab.gen_er(spec["n"], spec["mean_degree"], spec["seed"])
    u = [0, 1, 2, 3, 5, 5, 5, 5, 4, 11]
    v = [1, 2, 3, 4, 6, 7, 8, 9, 9, 12]
    return ab.csr_from_edges(13, np.array(u), np.array(v))


def graph_checksum(g) -> int:
    rp = g.rowptr.astype(np.uint64)
    col = g.col.astype(np.uint64)
    idx = np.arange(col.shape[0], dtype=np.uint64)
    return int((np.sum(rp * np.uint64(2654435761)) + np.sum((col + np.uint64(1)) * (idx % np.uint64(1009) + np.uint64(1)))) % np.uint64(2**61 - 1))


@pytest.fixture(scope="session")
def rmat16():
    """Config 0: RMAT scale 16, edgefactor 16 (A/B/C/D = .57/.19/.19/.05), 64 seeded roots."""
    import albba_gb300 as ab
    g = ab.gen_rmat(16, 16, seed=2024)
    roots = g.pick_roots(64, seed=7)
    return g, roots

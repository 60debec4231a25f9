"""The bounds-checked build and deterministic replays.

libalbba_gb300_checked.so (-DALB_CHECKED) checks every vertex id the
traversal kernels load -- SELL columns, push and long-row lists, frontier
queues -- before it is used as an index, and reports a bad one as
ALB_ERR_DEVICE instead of reading or writing out of bounds (no trap). The
single-root and 64-root parity suites, run on that build against the oracle,
must pass unchanged: no check fires on valid graphs and the checks change no
result. The reference has no such build (its only checks are allocation
failures, bfs/src/utils.c:102-109)."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_parity_suites_on_the_bounds_checked_build():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    lib = ge._build_module().build_library(checked=True)
    assert lib.exists()
    env = dict(os.environ, ALB_LIBRARY="checked")
    r = subprocess.run(
        [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
         "-k", "not full_scale and not injected",
         str(ROOT / "tests" / "test_bfs_gpu.py"), str(ROOT / "tests" / "test_msbfs_gpu.py"),
         str(ROOT / "tests" / "test_bypass_gpu.py")],
        env=env, cwd=ROOT, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and "failed" not in r.stdout
    # the subprocess really ran the checked library
    probe = subprocess.run(
        [sys.executable, "-c", "import albba_gb300 as ab; print(ab.LIB_PATH.name)"],
        env=env, cwd=ROOT, capture_output=True, text=True)
    assert probe.stdout.strip() == "libalbba_gb300_checked.so"


_STABLE = ("dir", "level", "nf", "mf", "nu", "mu", "active_slices", "bytes", "words_bypassed",
           "rows_scanned", "groups_read", "groups_bypassed", "edges_bypassed")


def _trace_key(dg):
    return [tuple(getattr(t, f) for f in _STABLE) for t in dg.level_trace()]


def test_deterministic_replays(rmat16):
    """Same graph, same root, same options: bit-identical levels, parents and
    per-level counters on every run (parents are fixed by the smallest-id
    rule, counters by the level sets)."""
    g, roots = rmat16
    with ab.Graph(g) as dg:
        dg.sell_build()
        for loop in ("host", "graph", "persistent"):
            for r in roots[:3]:
                runs = []
                for _ in range(3):
                    lv, pa, st = dg.bfs(int(r), ab.bfs_opts("beamer", loop, trace=True))
                    runs.append((lv, pa, st.num_levels, st.reached, st.edges, _trace_key(dg)))
                for other in runs[1:]:
                    assert np.array_equal(runs[0][0], other[0])
                    assert np.array_equal(runs[0][1], other[1])
                    assert runs[0][2:] == other[2:]
        outs = []
        for _ in range(3):
            lv, st = dg.msbfs64(roots, ab.bfs_opts("beamer", "host", trace=True))
            outs.append((lv, st.reached, st.edges, st.pushed_roots, _trace_key(dg)))
        for other in outs[1:]:
            assert np.array_equal(outs[0][0], other[0])
            assert outs[0][1:] == other[1:]

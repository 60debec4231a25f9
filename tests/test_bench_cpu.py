"""bench.py's contract pieces that run without a GPU: the reference arm's
JSON line (the oracle port timed on the host cores, small graph), the
non-zero ranks of a multi-rank reference run, and the roofline record built
from a level trace."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _run(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    env.setdefault("OMP_NUM_THREADS", "2")
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True,
                          text=True, env=env, timeout=300)


def test_reference_arm_json_line():
    p = _run(["--impl", "reference", "--scale", "12", "--steps", "2", "--warmup", "1"])
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["unit"] == "GTEPS" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"].startswith("RMAT scale 12")
    # the reference's own SELL and task settings, not the GPU arm's
    assert line["config"]["C"] == 256 and line["config"]["sigma"] == 16384
    assert line["config"]["tasks_per_level"] == 8


def test_reference_arm_other_ranks_do_nothing():
    p = _run(["--impl", "reference", "--scale", "12", "--steps", "1", "--warmup", "1"],
             {"RANK": "1", "WORLD_SIZE": "2"})
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


class _Rec:
    def __init__(self, level, d, byts, us):
        self.level, self.dir, self.bytes, self.step_us = level, d, byts, us


class _Graph:
    def __init__(self, trace):
        self.trace = trace

    def msbfs64_device(self, *a, **k):
        pass

    def level_trace(self):
        return self.trace


def test_roofline_record_from_trace():
    import albba_gb300 as ab
    trace = [_Rec(0, ab.DIR_TOPDOWN, 10, 50.0), _Rec(1, ab.DIR_TOPDOWN, 10, 400.0),
             _Rec(2, ab.DIR_BOTTOMUP, 2_800_000_000, 930.0), _Rec(3, ab.DIR_BOTTOMUP, 750_000_000, 260.0),
             _Rec(4, ab.DIR_TOPDOWN, 10, 50.0)]
    r = bench.roofline(_Graph(trace), None, None, "beamer")
    assert r["launches"] == 2
    assert r["bytes_per_launch"] == (2_800_000_000 + 750_000_000) / 2
    assert r["achieved"] == pytest.approx((2_800_000_000 + 750_000_000) / 1190.0 / 1e3)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    # DRAM traffic needs ncu: the bench run does not claim it
    assert r["traffic"] is None

"""Host-side checks that need no GPU: the C ABI exports, the generators and
graph file formats, and error reporting."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
from conftest import ROOT

HEADERS = sorted((ROOT / "include").glob("*.h"))
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b((?:alb|run_custom|print_additional|bfs_gb300)\w*)\s*\(", re.M)


def declared(header: Path) -> set[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return {m.group(1) for m in DECL.finditer(text)}


def test_every_declared_symbol_is_exported():
    import __graft_entry__ as ge
    build = ge._build_module()
    libs = {"albba.h": build.LIB, "albba_gen.h": build.LIB}
    seen = 0
    for h in HEADERS:
        names = declared(h)
        path = libs.get(h.name, build.PLUGIN if "plugin" in h.name else build.LIB)
        if not path.exists():
            pytest.fail(f"{path} missing")
        lib = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
        for name in sorted(names):
            assert hasattr(lib, name), f"{name} declared in {h.name} but not exported by {path.name}"
            seen += 1
    assert seen >= 20


def test_python_binding_lists_all_core_symbols():
    names = declared(ROOT / "include" / "albba.h") | declared(ROOT / "include" / "albba_gen.h")
    assert set(ab.EXPORTED) <= names | {"alb_selector_load", "alb_selector_clear"}


def _check_csr(g: ab.Csr):
    rp, col = g.rowptr, g.col
    assert rp[0] == 0 and np.all(np.diff(rp) >= 0) and rp[-1] == col.shape[0]
    n = g.n
    assert col.min(initial=0) >= 0 and col.max(initial=0) < n
    src = np.repeat(np.arange(n), np.diff(rp))
    assert not np.any(src == col), "self-loop"
    # rows strictly ascending (sorted, no duplicates)
    same_row = src[1:] == src[:-1]
    assert np.all(col[1:][same_row] > col[:-1][same_row])
    # symmetric
    fwd = src.astype(np.int64) * n + col
    bwd = col.astype(np.int64) * n + src
    assert np.array_equal(np.sort(fwd), np.sort(bwd))


def test_rmat_generator_is_deterministic_and_canonical():
    a = ab.gen_rmat(12, 16, seed=5)
    b = ab.gen_rmat(12, 16, seed=5)
    c = ab.gen_rmat(12, 16, seed=6)
    assert np.array_equal(a.rowptr, b.rowptr) and np.array_equal(a.col, b.col)
    assert not np.array_equal(a.col, c.col)
    _check_csr(a)
    assert a.n == 4096
    # edge factor 16: at most 2 * 16 * n directed entries after symmetrising
    assert 0.5 * 32 * a.n < a.nnz <= 32 * a.n
    deg = a.degrees()
    assert deg.max() > 20 * deg.mean()  # RMAT skew


def test_rmat_quadrant_probabilities():
    # no permutation: with a = 1 every edge is (0, 0) -> only self-loops -> empty graph
    g = ab.gen_rmat(8, 4, seed=1, a=1.0, b=0.0, c=0.0, permute=False)
    assert g.nnz == 0
    # a = 0, b = 1: every edge is (0, 2^s - 1)
    g = ab.gen_rmat(8, 4, seed=1, a=0.0, b=1.0, c=0.0, permute=False)
    assert g.nnz == 2 and set(g.col.tolist()) == {0, 255}


def test_grid_and_er_generators():
    g = ab.gen_grid(30, 20, drop=0.0, shortcut_frac=0.0, seed=1)
    _check_csr(g)
    assert g.nnz == 2 * (30 * 19 + 29 * 20)
    g2 = ab.gen_grid(30, 20, drop=0.1, shortcut_frac=0.01, seed=1)
    _check_csr(g2)
    assert g2.nnz < 2 * (30 * 19 + 29 * 20) + 2 * 6
    e = ab.gen_er(5000, 8.0, seed=3)
    _check_csr(e)
    assert abs(e.nnz / e.n - 8.0) < 0.5


def test_pick_roots_have_degree():
    g = ab.gen_rmat(12, 16, seed=5)
    r = g.pick_roots(64, seed=9)
    assert len(set(r.tolist())) == 64
    assert np.all(g.degrees()[r] >= 1)
    assert np.array_equal(r, g.pick_roots(64, seed=9))


def test_cbd_round_trip_and_corruption(tmp_path):
    g = ab.gen_rmat(10, 8, seed=4)
    p = tmp_path / "g.cbd"
    g.write_cbd(p)
    h = ab.read_cbd(p)
    assert np.array_equal(g.rowptr, h.rowptr) and np.array_equal(g.col, h.col)
    raw = p.read_bytes()
    # layout of bfs/src/biio.h:21-71: 3 ints, rowptr, col, fp64 values
    assert len(raw) == 12 + 4 * (g.n + 1) + 12 * g.nnz
    (tmp_path / "short.cbd").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(ab.AlbError) as ei:
        ab.read_cbd(tmp_path / "short.cbd")
    assert ei.value.code == ab.ERR_IO
    with pytest.raises(ab.AlbError) as ei:
        ab.read_cbd(tmp_path / "missing.cbd")
    assert ei.value.code == ab.ERR_IO
    bad = bytearray(raw)
    bad[12 + 4 * (g.n + 1): 12 + 4 * (g.n + 1) + 4] = (10**6).to_bytes(4, "little")
    (tmp_path / "bad.cbd").write_bytes(bytes(bad))
    with pytest.raises(ab.AlbError):
        ab.read_cbd(tmp_path / "bad.cbd")


def test_invalid_arguments_are_reported_not_fatal():
    with pytest.raises(ab.AlbError) as ei:
        ab.gen_rmat(0, 16)
    assert ei.value.code == ab.ERR_INVALID and "alb_gen_rmat" in ab.last_error()
    with pytest.raises(ab.AlbError):
        ab.csr_from_edges(4, np.array([0, 9]), np.array([1, 2]))
    h = C.c_void_p()
    # offsets not starting at 0 are refused on the host, before any device
    # work (the remaining checks run on the device: tests/test_ingest_gpu.py)
    rp = np.array([1, 1], np.int64)
    col = np.array([0], np.int32)
    code = ab.lib().alb_graph_create(1, rp.ctypes.data, col.ctypes.data, ab.CSR_SYMMETRIC, C.byref(h))
    assert code == ab.ERR_INVALID and not h.value
    rp = np.array([0, 1], np.int64)
    code = ab.lib().alb_graph_create(0, rp.ctypes.data, col.ctypes.data, 0, C.byref(h))
    assert code == ab.ERR_INVALID
    assert ab.lib().alb_bfs(None, 0, None, None, None, None) == ab.ERR_INVALID
    assert ab.lib().alb_sell_build(None, None, None) == ab.ERR_INVALID


def test_version_string():
    assert "sm_103a" in ab.version()

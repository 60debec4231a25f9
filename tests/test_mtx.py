"""Graph load from files (CPU): the Matrix Market reader and the undirected
conversion against the reference's own reader and driver code, through the
golden records of tests/golden/make_golden_mtx.py and, where the reference
tree is present, directly on further seeded files."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
RECS = json.loads((GOLDEN / "mtx.json").read_text())


def _csr_equal(g, rowptr, col):
    return (np.array_equal(g.rowptr, np.asarray(rowptr, np.int64))
            and np.array_equal(g.col, np.asarray(col, np.int32)))


@pytest.mark.parametrize("rec", RECS, ids=lambda r: r["name"])
def test_mtx_read_matches_reference(rec):
    g, sym = ab.read_mtx(GOLDEN / rec["file"])
    assert g.n == rec["n"]
    assert sym == bool(rec["symmetric"])
    assert _csr_equal(g, rec["rowptr"], rec["col"])


@pytest.mark.parametrize("rec", [r for r in RECS if not r["symmetric"]], ids=lambda r: r["name"])
def test_undirected_matches_reference(rec):
    g, _ = ab.read_mtx(GOLDEN / rec["file"])
    u = ab.csr_undirected(g)
    assert _csr_equal(u, rec["undirected_rowptr"], rec["undirected_col"])


@pytest.mark.parametrize("rec", RECS, ids=lambda r: r["name"])
def test_graph_read_is_the_driver_load(rec):
    g = ab.read_graph(GOLDEN / rec["file"])
    if rec["symmetric"]:
        assert _csr_equal(g, rec["rowptr"], rec["col"])
    else:
        assert _csr_equal(g, rec["undirected_rowptr"], rec["undirected_col"])


def test_graph_read_cbd(tmp_path):
    g = ab.gen_rmat(8, 8, seed=3)
    p = tmp_path / "g.cbd"
    g.write_cbd(p)
    h = ab.read_graph(p)
    assert np.array_equal(h.rowptr, g.rowptr) and np.array_equal(h.col, g.col)


def test_undirected_of_sorted_rows_is_the_union():
    # on ascending rows the merge is the sorted, duplicate-free union A | A^T
    g = ab.gen_er(300, 3.0, seed=4)
    rng = np.random.default_rng(5)
    keep = rng.random(g.nnz) < 0.5  # drop entries at random: a directed graph
    rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))[keep]
    cols = g.col[keep]
    rp = np.zeros(g.n + 1, np.int64)
    np.add.at(rp, rows + 1, 1)
    d = ab.Csr(np.cumsum(rp), cols.astype(np.int32))
    u = ab.csr_undirected(d)
    for i in range(g.n):
        want = np.union1d(cols[rows == i], rows[cols == i])
        assert np.array_equal(u.col[u.rowptr[i]:u.rowptr[i + 1]], want)


@pytest.mark.parametrize("text,code", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", ab.ERR_UNSUPPORTED),
    ("%%MatrixMarket matrix coordinate pattern general\n2 3 1\n1 1\n", ab.ERR_UNSUPPORTED),
    ("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n3 1\n", ab.ERR_IO),
    ("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n0 1\n", ab.ERR_IO),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", ab.ERR_IO),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 2\n", ab.ERR_IO),
    ("%%MatrixMarket matrix coordinate quaternion general\n2 2 0\n", ab.ERR_IO),
    ("%%MatrixMarket vector coordinate real general\n2 2 0\n", ab.ERR_IO),
    ("not a matrix market file\n", ab.ERR_IO),
    ("", ab.ERR_IO),
], ids=["array", "non-square", "row-out-of-range", "zero-index", "truncated", "missing-value",
        "bad-type", "bad-object", "no-banner", "empty-file"])
def test_malformed_files_refused(tmp_path, text, code):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    with pytest.raises(ab.AlbError) as ei:
        ab.read_mtx(p)
    assert ei.value.code == code


def test_unknown_extension_refused(tmp_path):
    p = tmp_path / "g.txt"
    p.write_text("1 2\n")
    with pytest.raises(ab.AlbError) as ei:
        ab.read_graph(p)
    assert ei.value.code == ab.ERR_UNSUPPORTED


def _ref():
    L = oracle.ref_lib()
    if L is None or not hasattr(L, "refh_mtx_info"):
        return None
    P = C.c_void_p
    L.refh_mtx_info.restype = C.c_int
    L.refh_mtx_info.argtypes = [C.c_char_p, P, P, P, P]
    L.refh_mtx_data.restype = C.c_int
    L.refh_mtx_data.argtypes = [C.c_char_p, C.c_int, C.c_int, P, P]
    L.refh_undirected.restype = C.c_int
    L.refh_undirected.argtypes = [C.c_int, P, P, P, P]
    return L


@pytest.mark.parametrize("seed", range(6))
def test_against_reference_code_directly(tmp_path, seed):
    # further seeded files through the reference's reader and merge (only
    # where the reference tree was compiled into oracle/_ref)
    L = _ref()
    if L is None:
        pytest.skip("reference tree not compiled here")
    import importlib.util
    spec = importlib.util.spec_from_file_location("mkg", GOLDEN / "make_golden_mtx.py")
    mkg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mkg)
    sym = ["general", "symmetric", "hermitian", "skew-symmetric"][seed % 4]
    typ = ["pattern", "real", "integer", "complex"][(seed // 2) % 4]
    p = tmp_path / "r.mtx"
    mkg.write_mtx(p, 20 + 7 * seed, 50 + 31 * seed, typ, sym, 100 + seed)
    info = np.zeros(4, np.int32)
    assert L.refh_mtx_info(str(p).encode(), info[0:].ctypes.data, info[1:].ctypes.data,
                           info[2:].ctypes.data, info[3:].ctypes.data) == 0
    rows, _, nnz, issym = (int(x) for x in info)
    rp = np.zeros(rows + 1, np.int32)
    col = np.zeros(max(nnz, 1), np.int32)
    assert L.refh_mtx_data(str(p).encode(), rows, nnz, rp.ctypes.data, col.ctypes.data) == 0
    g, s = ab.read_mtx(p)
    assert s == bool(issym)
    assert _csr_equal(g, rp, col[:nnz])
    urp = np.zeros(rows + 1, np.int32)
    ucol = np.zeros(max(2 * nnz, 1), np.int32)
    k = L.refh_undirected(rows, rp.ctypes.data, col.ctypes.data, urp.ctypes.data, ucol.ctypes.data)
    assert _csr_equal(ab.csr_undirected(g), urp, ucol[:k])

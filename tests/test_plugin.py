"""The drop-in BFS variant (libbfs_gb300.so) behind the reference's plugin
interface run_custom_bfs_test (bfs/src/bfs.h:13-24)."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import albba_gb300 as ab
import oracle
from conftest import ROOT

PLUGIN = ROOT / "albba_gb300" / "libbfs_gb300.so"
_REF_ROOT = oracle.reference_root()
REF_SRC = (_REF_ROOT / "bfs" / "src") if _REF_ROOT else Path("/nonexistent")


class SparseMatrixCSR(C.Structure):
    # layout of bfs/src/sparse_matrix.h:18-28
    _fields_ = [("name", C.c_char_p), ("values", C.POINTER(C.c_double)),
                ("column_indices", C.POINTER(C.c_int)), ("row_pointers", C.POINTER(C.c_int)),
                ("nrows", C.c_int), ("ncolumns", C.c_int), ("nnz", C.c_int),
                ("isSymmetric", C.c_int)]


def plugin():
    lib = C.CDLL(str(PLUGIN))
    lib.run_custom_bfs_test.restype = None
    lib.run_custom_bfs_test.argtypes = [C.POINTER(SparseMatrixCSR), C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_bool, C.c_bool]
    lib.bfs_gb300_last_levels.restype = C.POINTER(C.c_int)
    lib.bfs_gb300_last_parents.restype = C.POINTER(C.c_int)
    return lib


def test_plugin_exports_the_variant_interface():
    lib = plugin()
    for name in ("run_custom_bfs_test", "print_additional_custom_report", "sigma_window",
                 "chunk_size", "num_blocks", "algorithm_version", "required_matrix_format",
                 "verify", "perf_analysis", "bypass_record", "align_size"):
        assert hasattr(lib, name), name
    assert C.c_char_p.in_dll(lib, "algorithm_version") is not None


@pytest.mark.skipif(not (REF_SRC / "main.c").exists() or shutil.which("gcc") is None,
                    reason="reference driver sources not present on this machine")
def test_reference_driver_links_against_the_plugin(tmp_path):
    """The reference's own main.c and support sources, unchanged, link with
    libbfs_gb300.so in place of bfs_SELLCSv2.c + bfs_par_kernels.c."""
    srcs = [REF_SRC / f for f in ("main.c", "sparse_matrix.c", "utils.c", "sorting_utils.c",
                                  "report_results.c", "mytimer.c")]
    exe = tmp_path / "bfs_GB300"
    r = subprocess.run(["gcc", "-O2", "-fopenmp", "-DUSE_OMP", "-w", f"-I{REF_SRC}", *map(str, srcs),
                        f"-L{PLUGIN.parent}", "-lbfs_gb300", "-lalbba_gb300",
                        f"-Wl,-rpath,{PLUGIN.parent}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()


def call(lib, g: ab.Csr, root: int = 0, verify: int = 1, perf: int = 0):
    n = g.n
    rp = g.rowptr.astype(np.int32)
    col = np.ascontiguousarray(g.col, dtype=np.int32)
    vals = np.ones(max(g.nnz, 1))
    m = SparseMatrixCSR(b"/golden/graph", vals.ctypes.data_as(C.POINTER(C.c_double)),
                        col.ctypes.data_as(C.POINTER(C.c_int)),
                        rp.ctypes.data_as(C.POINTER(C.c_int)), n, n, g.nnz, 1)
    bfs_x = np.zeros(n)
    colidx_x = np.zeros(n, np.int32)
    colidx_x[0] = root
    bfs_x[root] = 1
    nnzx = np.array([1], np.int32)
    frontier = np.zeros(n, np.int32)
    num_vex = np.array([1], np.int32)
    conv = np.zeros(1)
    iters = np.zeros(n)
    bt = np.zeros(1)
    ni = np.zeros(1, np.int32)
    C.c_int.in_dll(lib, "verify").value = verify
    C.c_int.in_dll(lib, "perf_analysis").value = perf
    lib.run_custom_bfs_test(C.byref(m), bfs_x.ctypes.data, colidx_x.ctypes.data, nnzx.ctypes.data,
                            frontier.ctypes.data, num_vex.ctypes.data, conv.ctypes.data,
                            iters.ctypes.data, bt.ctypes.data, ni.ctypes.data, True, False)
    return dict(frontier=frontier[: ni[0]], num_vex=int(num_vex[0]), conv=conv[0],
                iter_times=iters[: ni[0]], bfs_time=bt[0], num_iter=int(ni[0]), nnzx=int(nnzx[0]))


@pytest.mark.gpu
@pytest.mark.parametrize("perf", [0, 1])
def test_plugin_matches_run_bfs_ref_counts(perf):
    lib = plugin()
    g = ab.gen_rmat(14, 16, seed=31)
    for root in g.pick_roots(4, 5):
        out = call(lib, g, int(root), verify=1, perf=perf)
        lv, pa, nl = oracle.bfs(g.rowptr, g.col, int(root))
        assert out["num_iter"] == nl
        assert out["frontier"].tolist() == oracle.level_counts(lv, nl).tolist()
        assert out["num_vex"] == int(np.count_nonzero(lv >= 0))
        assert out["bfs_time"] > 0 and out["conv"] > 0 and out["nnzx"] == 0
        if perf:
            assert np.all(out["iter_times"] > 0)
        got = np.ctypeslib.as_array(lib.bfs_gb300_last_levels(), shape=(g.n,))
        gotp = np.ctypeslib.as_array(lib.bfs_gb300_last_parents(), shape=(g.n,))
        assert np.array_equal(got, lv) and np.array_equal(gotp, pa)


@pytest.mark.gpu
def test_plugin_writes_bypass_records(tmp_path, monkeypatch):
    """bypass_record = 1: one line per run in the reference's slice- and
    column-bypass CSV files (bfs/src/bfs_SELLCSv2.c:773-818), its counts the
    kernels' per-level bypass statistics."""
    lib = plugin()
    g = ab.gen_rmat(14, 16, seed=31)
    monkeypatch.setenv("ALB_BYPASS_DIR", str(tmp_path))
    C.c_int.in_dll(lib, "bypass_record").value = 1
    try:
        out = call(lib, g, 0, verify=1)
    finally:
        C.c_int.in_dll(lib, "bypass_record").value = 0
    for fname in ("bfs-slice-bypass.csv", "bfs-column-bypass.csv"):
        line = (tmp_path / fname).read_text().strip().split(",")
        assert line[0] == "graph" and int(line[1]) == g.n and int(line[3]) == g.nnz
        assert int(line[4]) == out["num_iter"]
        counts = [int(x) for x in line[6:]]
        assert len(counts) == out["num_iter"] and all(c >= 0 for c in counts)
    slices = [int(x) for x in (tmp_path / "bfs-slice-bypass.csv").read_text().split(",")[6:]]
    # the levels after the largest pull skip fully visited words
    assert sum(slices) > 0

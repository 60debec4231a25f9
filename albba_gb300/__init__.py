"""albba_gb300: GB300-native linear-algebra BFS (Python binding over the C ABI).

The native library ``libalbba_gb300.so`` (built in-tree by
``albba_gb300.build.build_library``) does all the work; this module only
marshals arguments through ctypes. There is no Python or CPU fallback: if the
library is missing, importing this package raises ImportError.

Reference mapping (scalbba/albba):
  run_custom_bfs_test (bfs/src/bfs.h:13-24)  ->  Graph.sell_build + Graph.bfs
  run_bfs_ref's per-level frontier counts     ->  Stats / Graph.level_trace
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
# ALB_LIBRARY=checked loads the bounds-checked build (tests of the kernels'
# index discipline), ALB_LIBRARY=<path to a .so> another build of the same
# ABI; the default is the production library
_sel = os.environ.get("ALB_LIBRARY", "")
LIB_PATH = (_PKG / "libalbba_gb300_checked.so" if _sel == "checked"
            else Path(_sel) if _sel.endswith(".so") else _PKG / "libalbba_gb300.so")

if not LIB_PATH.exists():
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
        "(there is no CPU fallback)")

_lib = C.CDLL(str(LIB_PATH), mode=C.RTLD_GLOBAL)

# ----------------------------------------------------------------- constants
OK = 0
ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_TIMEOUT = -1, -2, -3, -4
ERR_STATE, ERR_IO, ERR_UNSUPPORTED, ERR_DEVICE = -5, -6, -7, -8

CSR_OUT, CSR_IN, CSR_SYMMETRIC, CSR_SORTED = 0, 1, 2, 4

POLICY_BEAMER, POLICY_REF004, POLICY_LEARNED = 0, 1, 2
POLICY_TOPDOWN, POLICY_BOTTOMUP, POLICY_BOTTOMUP_NOBYPASS = 3, 4, 5
POLICIES = {"beamer": 0, "ref004": 1, "learned": 2, "topdown": 3, "bottomup": 4,
            "bottomup_nobypass": 5}

LOOP_HOST, LOOP_GRAPH, LOOP_PERSISTENT = 0, 1, 2
LOOPS = {"host": 0, "graph": 1, "persistent": 2}

DIR_TOPDOWN, DIR_BOTTOMUP, DIR_BOTTOMUP_NOBYPASS = 0, 1, 2

EXPORTED = [
    "alb_last_error", "alb_version", "alb_graph_create", "alb_graph_create32",
    "alb_graph_destroy", "alb_graph_info", "alb_graph_set_stream", "alb_sell_opts_default", "alb_sell_build",
    "alb_sell_export", "alb_sell_long_export", "alb_bfs_opts_default", "alb_bfs", "alb_bfs_device",
    "alb_level_trace", "alb_debug_fail_alloc_after", "alb_gen_rmat", "alb_gen_grid",
    "alb_gen_er", "alb_csr_from_edges", "alb_pick_roots", "alb_host_csr_free",
    "alb_cbd_write", "alb_cbd_read", "alb_mtx_read", "alb_csr_undirected", "alb_graph_read",
    "alb_selector_load", "alb_selector_clear",
    "alb_msbfs64", "alb_msbfs64_device", "alb_bfs_profile", "alb_msbfs64_profile",
    "alb_mlp_forward", "alb_mlp_loss_grad", "alb_adam_step", "alb_selector_train",
    "alb_worklist_create", "alb_worklist_destroy", "alb_worklist_add", "alb_worklist_size",
    "alb_worklist_run", "alb_worklist_run_device",
]


class AlbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"albba_gb300 error {code}: {msg}")
        self.code = code


# ------------------------------------------------------------------- structs
class SellOpts(C.Structure):
    _fields_ = [("C", C.c_int32), ("sigma", C.c_int32), ("long_row", C.c_int32)]


class BfsOpts(C.Structure):
    _fields_ = [("policy", C.c_int32), ("loop", C.c_int32), ("alpha", C.c_float),
                ("beta", C.c_float), ("block", C.c_int32), ("trace", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("num_levels", C.c_int32), ("levels_topdown", C.c_int32),
                ("levels_bottomup", C.c_int32), ("pushed_roots", C.c_int32),
                ("reached", C.c_int64), ("edges", C.c_int64), ("ms", C.c_double),
                ("kernels", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class LevelRec(C.Structure):
    _fields_ = [("dir", C.c_int32), ("level", C.c_int32), ("nf", C.c_int64), ("mf", C.c_int64),
                ("nu", C.c_int64), ("mu", C.c_int64), ("active_slices", C.c_int64),
                ("t_ns", C.c_int64), ("bytes", C.c_int64), ("step_us", C.c_float),
                ("pad_", C.c_int32), ("words_bypassed", C.c_int64), ("rows_scanned", C.c_int64),
                ("groups_read", C.c_int64), ("groups_bypassed", C.c_int64),
                ("edges_bypassed", C.c_int64)]


class LevelProfile(C.Structure):
    _fields_ = [("rec", LevelRec), ("feat", C.c_float * 8), ("us", C.c_float * 3),
                ("best", C.c_int32)]


class HostCsr(C.Structure):
    _fields_ = [("n", C.c_int64), ("nnz", C.c_int64), ("rowptr", C.POINTER(C.c_int64)),
                ("col", C.POINTER(C.c_int32))]


_P = C.c_void_p
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)

_sigs = {
    "alb_last_error": (C.c_char_p, []),
    "alb_version": (C.c_char_p, []),
    "alb_graph_create": (C.c_int32, [C.c_int64, _P, _P, C.c_uint32, C.POINTER(_P)]),
    "alb_graph_create32": (C.c_int32, [C.c_int32, _P, _P, C.c_uint32, C.POINTER(_P)]),
    "alb_graph_create_undirected": (C.c_int32, [C.c_int64, _P, _P, C.POINTER(_P)]),
    "alb_graph_load": (C.c_int32, [C.c_char_p, C.POINTER(_P)]),
    "alb_graph_export_csr": (C.c_int32, [_P, C.c_int32, _P, _P]),
    "alb_graph_is_symmetric": (C.c_int32, [_P, _i32p]),
    "alb_graph_destroy": (None, [_P]),
    "alb_graph_info": (C.c_int32, [_P, _i64p, _i64p]),
    "alb_graph_set_stream": (C.c_int32, [_P, _P]),
    "alb_sell_opts_default": (None, [C.POINTER(SellOpts)]),
    "alb_sell_build": (C.c_int32, [_P, C.POINTER(SellOpts), C.POINTER(C.c_double)]),
    "alb_sell_export": (C.c_int32, [_P, _i64p, _P, _P, _P, _P]),
    "alb_sell_long_export": (C.c_int32, [_P, _i64p, _P, _P, _P]),
    "alb_bfs_opts_default": (None, [C.POINTER(BfsOpts)]),
    "alb_bfs": (C.c_int32, [_P, C.c_int32, C.POINTER(BfsOpts), _P, _P, C.POINTER(Stats)]),
    "alb_bfs_device": (C.c_int32, [_P, C.c_int32, C.POINTER(BfsOpts), _P, _P, C.POINTER(Stats)]),
    "alb_level_trace": (C.c_int32, [_P, C.c_int32, C.POINTER(LevelRec), _i32p]),
    "alb_debug_fail_alloc_after": (None, [C.c_int32]),
    "alb_debug_device_waits": (None, [C.c_int32, C.c_int32, C.c_int32, C.c_int64]),
    "alb_gen_rmat": (C.c_int32, [C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                 C.c_double, C.c_int32, C.POINTER(HostCsr)]),
    "alb_gen_grid": (C.c_int32, [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_uint64,
                                 C.POINTER(HostCsr)]),
    "alb_gen_er": (C.c_int32, [C.c_int64, C.c_double, C.c_uint64, C.POINTER(HostCsr)]),
    "alb_csr_from_edges": (C.c_int32, [C.c_int64, C.c_int64, _P, _P, C.POINTER(HostCsr)]),
    "alb_pick_roots": (C.c_int32, [C.POINTER(HostCsr), C.c_int32, C.c_uint64, _P]),
    "alb_host_csr_free": (None, [C.POINTER(HostCsr)]),
    "alb_cbd_write": (C.c_int32, [C.c_char_p, C.POINTER(HostCsr)]),
    "alb_cbd_read": (C.c_int32, [C.c_char_p, C.POINTER(HostCsr)]),
    "alb_mtx_read": (C.c_int32, [C.c_char_p, C.POINTER(HostCsr), _i32p]),
    "alb_csr_undirected": (C.c_int32, [C.POINTER(HostCsr), C.POINTER(HostCsr)]),
    "alb_graph_read": (C.c_int32, [C.c_char_p, C.POINTER(HostCsr)]),
    "alb_msbfs64": (C.c_int32, [_P, _P, C.c_int32, C.POINTER(BfsOpts), _P, C.POINTER(Stats)]),
    "alb_msbfs64_device": (C.c_int32, [_P, _P, C.c_int32, C.POINTER(BfsOpts), _P,
                                       C.POINTER(Stats)]),
    "alb_bfs_profile": (C.c_int32, [_P, C.c_int32, C.POINTER(BfsOpts), C.c_int32,
                                    C.POINTER(LevelProfile), _i32p]),
    "alb_msbfs64_profile": (C.c_int32, [_P, _P, C.c_int32, C.POINTER(BfsOpts), C.c_int32,
                                        C.POINTER(LevelProfile), _i32p]),
    "alb_mlp_forward": (C.c_int32, [_P, _P, C.c_int32, _P]),
    "alb_mlp_loss_grad": (C.c_int32, [_P, _P, _P, _P, C.c_int32, _P, C.POINTER(C.c_float)]),
    "alb_adam_step": (C.c_int32, [_P, _P, _P, _P, C.c_int32, C.c_float, C.c_float, C.c_float,
                                  C.c_float]),
    "alb_selector_train": (C.c_int32, [_P, _P, _P, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                       C.c_int32, _P, C.POINTER(C.c_float)]),
    "alb_worklist_create": (C.c_int32, [C.POINTER(_P)]),
    "alb_worklist_destroy": (None, [_P]),
    "alb_worklist_add": (C.c_int32, [_P, _P, _P, C.c_int32, C.c_float, C.c_float]),
    "alb_worklist_size": (C.c_int32, [_P, _i64p, _i32p]),
    "alb_worklist_run": (C.c_int32, [_P, C.c_int32, _P, C.POINTER(Stats)]),
    "alb_worklist_run_device": (C.c_int32, [_P, C.c_int32, _P, C.POINTER(Stats)]),
    "alb_selector_load": (C.c_int32, [C.c_int32, _P]),
    "alb_selector_clear": (C.c_int32, [C.c_int32]),
    "alb_spmspv_merge": (C.c_int32, [_P, _P, C.c_int64, _P, _P, _i64p]),
    "alb_sellmat_create": (C.c_int32, [C.c_int64, _P, _P, _P, C.c_int32, C.POINTER(_P)]),
    "alb_sellmat_destroy": (None, [_P]),
    "alb_sellmat_info": (C.c_int32, [_P, _i64p, _i64p, _i64p]),
    "alb_sellmat_spmv": (C.c_int32, [_P, _P, _P, C.POINTER(C.c_float)]),
    "alb_sellmat_spmv_host": (C.c_int32, [_P, _P, _P]),
}
for _name, (_res, _args) in _sigs.items():
    _f = getattr(_lib, _name)
    _f.restype = _res
    _f.argtypes = _args


def lib() -> C.CDLL:
    return _lib


def last_error() -> str:
    return _lib.alb_last_error().decode()


def version() -> str:
    return _lib.alb_version().decode()


def check(code: int) -> None:
    if code != OK:
        raise AlbError(code, last_error())


def _ptr(a) -> int | None:
    """Address of a numpy array or a torch tensor (None passes through)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


# ---------------------------------------------------------------- host CSR
class Csr:
    """Host CSR: int64 row offsets, int32 columns (numpy)."""

    def __init__(self, rowptr: np.ndarray, col: np.ndarray, _owner: HostCsr | None = None):
        self.rowptr = rowptr
        self.col = col
        self._owner = _owner

    @property
    def n(self) -> int:
        return int(self.rowptr.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def degrees(self) -> np.ndarray:
        return np.diff(self.rowptr)

    def _as_host(self) -> HostCsr:
        h = HostCsr()
        h.n = self.n
        h.nnz = self.nnz
        h.rowptr = self.rowptr.ctypes.data_as(_i64p)
        h.col = self.col.ctypes.data_as(_i32p)
        return h

    def __del__(self):
        if self._owner is not None:
            _lib.alb_host_csr_free(C.byref(self._owner))
            self._owner = None

    def pick_roots(self, count: int, seed: int) -> np.ndarray:
        roots = np.empty(count, dtype=np.int32)
        h = self._as_host()
        check(_lib.alb_pick_roots(C.byref(h), count, seed, roots.ctypes.data))
        return roots

    def write_cbd(self, path: str | os.PathLike) -> None:
        h = self._as_host()
        check(_lib.alb_cbd_write(str(path).encode(), C.byref(h)))


def _wrap(h: HostCsr) -> Csr:
    n, nnz = h.n, h.nnz
    rp = np.ctypeslib.as_array(h.rowptr, shape=(n + 1,))
    col = np.ctypeslib.as_array(h.col, shape=(max(nnz, 1),))[:nnz]
    return Csr(rp, col, _owner=h)


def gen_rmat(scale: int, edgefactor: int = 16, seed: int = 1, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, permute: bool = True) -> Csr:
    h = HostCsr()
    check(_lib.alb_gen_rmat(scale, edgefactor, seed, a, b, c, 1 if permute else 0, C.byref(h)))
    return _wrap(h)


def gen_grid(rows: int, cols: int, drop: float = 0.1, shortcut_frac: float = 1e-4,
             seed: int = 1) -> Csr:
    h = HostCsr()
    check(_lib.alb_gen_grid(rows, cols, drop, shortcut_frac, seed, C.byref(h)))
    return _wrap(h)


def gen_er(n: int, mean_degree: float = 8.0, seed: int = 1) -> Csr:
    h = HostCsr()
    check(_lib.alb_gen_er(n, mean_degree, seed, C.byref(h)))
    return _wrap(h)


def csr_from_edges(n: int, u: np.ndarray, v: np.ndarray) -> Csr:
    u = np.ascontiguousarray(u, dtype=np.int32)
    v = np.ascontiguousarray(v, dtype=np.int32)
    h = HostCsr()
    check(_lib.alb_csr_from_edges(n, u.shape[0], u.ctypes.data, v.ctypes.data, C.byref(h)))
    return _wrap(h)


def read_cbd(path: str | os.PathLike) -> Csr:
    h = HostCsr()
    check(_lib.alb_cbd_read(str(path).encode(), C.byref(h)))
    return _wrap(h)


def read_mtx(path: str | os.PathLike) -> tuple[Csr, bool]:
    """Matrix Market file -> (CSR as the reference's reader builds it,
    symmetric flag); see alb_mtx_read."""
    h = HostCsr()
    sym = C.c_int32()
    check(_lib.alb_mtx_read(str(path).encode(), C.byref(h), C.byref(sym)))
    return _wrap(h), bool(sym.value)


def csr_undirected(g: Csr) -> Csr:
    """The reference driver's undirected conversion (alb_csr_undirected)."""
    src = g._as_host()
    h = HostCsr()
    check(_lib.alb_csr_undirected(C.byref(src), C.byref(h)))
    return _wrap(h)


def read_graph(path: str | os.PathLike) -> Csr:
    """Graph load of the reference driver: .cbd as is, .mtx made undirected
    unless symmetric (alb_graph_read)."""
    h = HostCsr()
    check(_lib.alb_graph_read(str(path).encode(), C.byref(h)))
    return _wrap(h)


# -------------------------------------------------------------- device graph
def bfs_opts(policy: str | int = "beamer", loop: str | int = "graph", alpha: float = 14.0,
             beta: float = 24.0, block: int = 256, trace: bool = False) -> BfsOpts:
    o = BfsOpts()
    _lib.alb_bfs_opts_default(C.byref(o))
    o.policy = POLICIES[policy] if isinstance(policy, str) else int(policy)
    o.loop = LOOPS[loop] if isinstance(loop, str) else int(loop)
    o.alpha, o.beta, o.block, o.trace = alpha, beta, block, 1 if trace else 0
    return o


@dataclass
class SellExport:
    nslices: int
    perm: np.ndarray
    width: np.ndarray
    slice_off: np.ndarray
    col: np.ndarray


class Graph:
    """A graph resident on the current CUDA device."""

    def __init__(self, csr: Csr, flags: int = CSR_SYMMETRIC):
        self._h = _P()
        rp = np.ascontiguousarray(csr.rowptr, dtype=np.int64)
        col = np.ascontiguousarray(csr.col, dtype=np.int32)
        check(_lib.alb_graph_create(csr.n, rp.ctypes.data, col.ctypes.data, flags,
                                    C.byref(self._h)))
        self.n = csr.n
        self.nnz = csr.nnz

    @classmethod
    def from_int32(cls, n: int, rowptr: np.ndarray, col: np.ndarray, flags: int) -> "Graph":
        g = cls.__new__(cls)
        g._h = _P()
        rp = np.ascontiguousarray(rowptr, dtype=np.int32)
        cc = np.ascontiguousarray(col, dtype=np.int32)
        check(_lib.alb_graph_create32(n, rp.ctypes.data, cc.ctypes.data, flags, C.byref(g._h)))
        g.n, g.nnz = n, int(rp[-1])
        return g

    @classmethod
    def _from_handle(cls, h: C.c_void_p) -> "Graph":
        g = cls.__new__(cls)
        g._h = h
        n, nnz = C.c_int64(), C.c_int64()
        check(_lib.alb_graph_info(h, C.byref(n), C.byref(nnz)))
        g.n, g.nnz = n.value, nnz.value
        return g

    @classmethod
    def undirected(cls, csr: Csr) -> "Graph":
        """The reference driver's undirected graph of csr, built on the device."""
        h = _P()
        rp = np.ascontiguousarray(csr.rowptr, dtype=np.int64)
        col = np.ascontiguousarray(csr.col, dtype=np.int32)
        check(_lib.alb_graph_create_undirected(csr.n, rp.ctypes.data, col.ctypes.data,
                                               C.byref(h)))
        return cls._from_handle(h)

    @classmethod
    def load(cls, path: str | os.PathLike) -> "Graph":
        """A .cbd or .mtx file as the reference driver loads it, onto the device."""
        h = _P()
        check(_lib.alb_graph_load(str(path).encode(), C.byref(h)))
        return cls._from_handle(h)

    def export_csr(self, side: int = 0) -> Csr:
        """The device CSR (side 0: pull side, 1: push side) copied to the host."""
        rp = np.empty(self.n + 1, np.int64)
        check(_lib.alb_graph_export_csr(self._h, side, rp.ctypes.data, None))
        col = np.empty(max(int(rp[-1]), 1), np.int32)
        check(_lib.alb_graph_export_csr(self._h, side, None, col.ctypes.data))
        return Csr(rp, col[: int(rp[-1])])

    def spmspv_merge(self, frontier, visited_bits) -> np.ndarray:
        """Ascending distinct unvisited out-neighbours of the frontier
        (alb_spmspv_merge); visited_bits: uint32 bitmap over original ids."""
        x = np.ascontiguousarray(frontier, dtype=np.int32)
        vb = np.ascontiguousarray(visited_bits, dtype=np.uint32)
        y = np.empty(self.n, np.int32)
        ny = C.c_int64()
        check(_lib.alb_spmspv_merge(self._h, x.ctypes.data, x.shape[0], vb.ctypes.data,
                                    y.ctypes.data, C.byref(ny)))
        return y[: ny.value]

    @property
    def symmetric(self) -> bool:
        s = C.c_int32()
        check(_lib.alb_graph_is_symmetric(self._h, C.byref(s)))
        return bool(s.value)

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.alb_graph_destroy(self._h)
            self._h = _P()

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def set_stream(self, cuda_stream: int | None) -> None:
        """Run on a caller stream (e.g. torch.cuda.current_stream().cuda_stream)."""
        check(_lib.alb_graph_set_stream(self._h, cuda_stream))

    def sell_build(self, C_: int = 32, sigma: int = 1024, long_row: int = 1024) -> float:
        """Build SELL-C-sigma on the device; returns the build time in ms."""
        o = SellOpts(C_, sigma, long_row)
        ms = C.c_double()
        check(_lib.alb_sell_build(self._h, C.byref(o), C.byref(ms)))
        return ms.value

    def sell_export(self) -> SellExport:
        ns = C.c_int64()
        check(_lib.alb_sell_export(self._h, C.byref(ns), None, None, None, None))
        perm = np.empty(self.n, np.int32)
        width = np.empty(ns.value, np.int32)
        off = np.empty(ns.value + 1, np.int64)
        check(_lib.alb_sell_export(self._h, None, None, None, off.ctypes.data, None))
        col = np.empty(int(off[-1]), np.int32)
        check(_lib.alb_sell_export(self._h, None, perm.ctypes.data, width.ctypes.data, None,
                                   col.ctypes.data))
        return SellExport(ns.value, perm, width, off, col)

    def sell_long_export(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        nl = C.c_int64()
        check(_lib.alb_sell_long_export(self._h, C.byref(nl), None, None, None))
        lrow = np.empty(max(nl.value, 1), np.int32)
        lptr = np.empty(nl.value + 1, np.int64)
        check(_lib.alb_sell_long_export(self._h, None, lrow.ctypes.data, lptr.ctypes.data, None))
        lcol = np.empty(max(int(lptr[-1]), 1), np.int32)
        check(_lib.alb_sell_long_export(self._h, None, None, None, lcol.ctypes.data))
        return lrow[: nl.value], lptr, lcol[: int(lptr[-1])]

    def bfs(self, root: int, opts: BfsOpts | None = None, want_level: bool = True,
            want_parent: bool = True) -> tuple[np.ndarray | None, np.ndarray | None, Stats]:
        lv = np.empty(self.n, np.int32) if want_level else None
        pa = np.empty(self.n, np.int32) if want_parent else None
        st = Stats()
        o = opts or bfs_opts()
        check(_lib.alb_bfs(self._h, int(root), C.byref(o), _ptr(lv), _ptr(pa), C.byref(st)))
        return lv, pa, st

    def bfs_device(self, root: int, d_level=None, d_parent=None,
                   opts: BfsOpts | None = None) -> Stats:
        st = Stats()
        o = opts or bfs_opts()
        check(_lib.alb_bfs_device(self._h, int(root), C.byref(o), _ptr(d_level), _ptr(d_parent),
                                  C.byref(st)))
        return st

    def msbfs64(self, roots, opts: BfsOpts | None = None,
                out: np.ndarray | None = None) -> tuple[np.ndarray, Stats]:
        """Levels from up to 64 roots at once: array (n, 64), column i = roots[i].
        out: a C-contiguous int32 (n, 64) host array to fill (page-locked
        memory is written by the device directly)."""
        r = np.ascontiguousarray(roots, dtype=np.int32)
        if out is None:
            out = np.empty((self.n, 64), np.int32)
        elif out.dtype != np.int32 or out.shape != (self.n, 64) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous int32 array of shape (n, 64)")
        st = Stats()
        o = opts or bfs_opts()
        check(_lib.alb_msbfs64(self._h, r.ctypes.data, r.shape[0], C.byref(o), out.ctypes.data,
                               C.byref(st)))
        return out, st

    def msbfs64_device(self, roots, d_levels=None, opts: BfsOpts | None = None) -> Stats:
        r = np.ascontiguousarray(roots, dtype=np.int32)
        st = Stats()
        o = opts or bfs_opts()
        check(_lib.alb_msbfs64_device(self._h, r.ctypes.data, r.shape[0], C.byref(o),
                                      _ptr(d_levels), C.byref(st)))
        return st

    def bfs_profile(self, root: int, opts: BfsOpts | None = None) -> list[LevelProfile]:
        """Per-level step times of all three variants (see alb_bfs_profile)."""
        o = opts or bfs_opts()
        cnt = C.c_int32()
        cap = 4096
        buf = (LevelProfile * cap)()
        check(_lib.alb_bfs_profile(self._h, int(root), C.byref(o), cap, buf, C.byref(cnt)))
        return list(buf[: min(cnt.value, cap)])

    def msbfs64_profile(self, roots, opts: BfsOpts | None = None) -> list[LevelProfile]:
        r = np.ascontiguousarray(roots, dtype=np.int32)
        o = opts or bfs_opts()
        cnt = C.c_int32()
        cap = 4096
        buf = (LevelProfile * cap)()
        check(_lib.alb_msbfs64_profile(self._h, r.ctypes.data, r.shape[0], C.byref(o), cap, buf,
                                       C.byref(cnt)))
        return list(buf[: min(cnt.value, cap)])

    def level_trace(self) -> list[LevelRec]:
        cnt = C.c_int32()
        check(_lib.alb_level_trace(self._h, 0, None, C.byref(cnt)))
        buf = (LevelRec * max(cnt.value, 1))()
        check(_lib.alb_level_trace(self._h, cnt.value, buf, C.byref(cnt)))
        return list(buf[: cnt.value])


class SellMatrix:
    """fp64 SELL-C-sigma matrix on the current device (y = A x)."""

    def __init__(self, rowptr, col, values, sigma: int = 1024):
        self._h = _P()
        rp = np.ascontiguousarray(rowptr, dtype=np.int64)
        cl = np.ascontiguousarray(col, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        self.n = rp.shape[0] - 1
        check(_lib.alb_sellmat_create(self.n, rp.ctypes.data, cl.ctypes.data, v.ctypes.data,
                                      sigma, C.byref(self._h)))
        nnz, stored = C.c_int64(), C.c_int64()
        check(_lib.alb_sellmat_info(self._h, None, C.byref(nnz), C.byref(stored)))
        self.nnz, self.stored = nnz.value, stored.value

    def spmv(self, x) -> np.ndarray:
        xx = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n, np.float64)
        check(_lib.alb_sellmat_spmv_host(self._h, xx.ctypes.data, y.ctypes.data))
        return y

    def spmv_device(self, d_x, d_y) -> float:
        """Device vectors (torch tensors or pointers); returns the kernel's microseconds."""
        us = C.c_float()
        check(_lib.alb_sellmat_spmv(self._h, _ptr(d_x), _ptr(d_y), C.byref(us)))
        return us.value

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.alb_sellmat_destroy(self._h)
            self._h = _P()

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Worklist:
    """Persistent multi-graph BFS (alb_worklist_*). Keeps its graphs alive."""

    def __init__(self):
        self._h = _P()
        check(_lib.alb_worklist_create(C.byref(self._h)))
        self._graphs: list[Graph] = []
        self._layout: list[tuple[int, int, int]] = []  # (graph index, root, n)

    def add(self, g: Graph, roots, alpha: float = 14.0, beta: float = 24.0) -> None:
        r = np.ascontiguousarray(roots, dtype=np.int32)
        check(_lib.alb_worklist_add(self._h, g.handle, r.ctypes.data, r.shape[0], alpha, beta))
        self._graphs.append(g)
        for x in r:
            self._layout.append((len(self._graphs) - 1, int(x), g.n))

    def size(self) -> tuple[int, int]:
        e, k = C.c_int64(), C.c_int32()
        check(_lib.alb_worklist_size(self._h, C.byref(e), C.byref(k)))
        return e.value, k.value

    def run(self, block: int = 256) -> tuple[list[np.ndarray], Stats]:
        total, _ = self.size()
        out = np.empty(max(total, 1), np.int32)
        st = Stats()
        check(_lib.alb_worklist_run(self._h, block, out.ctypes.data, C.byref(st)))
        res, off = [], 0
        for _, _, n in self._layout:
            res.append(out[off: off + n])
            off += n
        return res, st

    def run_device(self, d_levels, block: int = 256) -> Stats:
        st = Stats()
        check(_lib.alb_worklist_run_device(self._h, block, _ptr(d_levels), C.byref(st)))
        return st

    @property
    def layout(self):
        return list(self._layout)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.alb_worklist_destroy(self._h)
            self._h = _P()

    def __del__(self):
        self.close()


NPARAM = 1443


def mlp_forward(params, x) -> np.ndarray:
    p = np.ascontiguousarray(params, np.float32)
    xx = np.ascontiguousarray(x, np.float32)
    out = np.empty((xx.shape[0], 3), np.float32)
    check(_lib.alb_mlp_forward(p.ctypes.data, xx.ctypes.data, xx.shape[0], out.ctypes.data))
    return out


def mlp_loss_grad(params, x, y, mask) -> tuple[float, np.ndarray]:
    p = np.ascontiguousarray(params, np.float32)
    xx, yy, mm = (np.ascontiguousarray(a, np.float32) for a in (x, y, mask))
    g = np.empty(NPARAM, np.float32)
    loss = C.c_float()
    check(_lib.alb_mlp_loss_grad(p.ctypes.data, xx.ctypes.data, yy.ctypes.data, mm.ctypes.data,
                                 xx.shape[0], g.ctypes.data, C.byref(loss)))
    return loss.value, g


def adam_step(params, grad, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8) -> None:
    """In place on params, m, v (float32 numpy arrays), on the GPU."""
    g = np.ascontiguousarray(grad, np.float32)
    check(_lib.alb_adam_step(params.ctypes.data, g.ctypes.data, m.ctypes.data, v.ctypes.data,
                             int(t), lr, b1, b2, eps))


def selector_train(x, y, mask, steps: int = 3000, lr: float = 3e-3, seed: int = 0,
                   params=None) -> tuple[np.ndarray, float]:
    """Full-batch Adam on the GPU; He init from seed unless params is given."""
    xx, yy, mm = (np.ascontiguousarray(a, np.float32) for a in (x, y, mask))
    p = np.zeros(NPARAM, np.float32) if params is None else np.array(params, np.float32)
    loss = C.c_float()
    check(_lib.alb_selector_train(xx.ctypes.data, yy.ctypes.data, mm.ctypes.data, xx.shape[0],
                                  steps, lr, seed, 1 if params is None else 0, p.ctypes.data,
                                  C.byref(loss)))
    return p, loss.value


def selector_load(which: int, params: np.ndarray) -> None:
    p = np.ascontiguousarray(params, dtype=np.float32)
    assert p.size == 1443
    check(_lib.alb_selector_load(which, p.ctypes.data))


def selector_clear(which: int) -> None:
    check(_lib.alb_selector_clear(which))


def debug_fail_alloc_after(k: int) -> None:
    _lib.alb_debug_fail_alloc_after(k)


def debug_device_waits(withhold_level: int = -1, withhold_block: int = 0, short_bulk: bool = False,
                       timeout_us: int = 0) -> None:
    """Test hooks of the bounded device waits (alb_debug_device_waits);
    no arguments: all off."""
    _lib.alb_debug_device_waits(withhold_level, withhold_block, 1 if short_bulk else 0, timeout_us)

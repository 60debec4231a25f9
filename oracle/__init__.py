"""CPU oracle for the ALBBA BFS hot path (ctypes over oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker (or the timed CPU
baseline), never by the albba_gb300 product. See oracle.h for what each
function restates from the reference, and tests/golden/ for the golden
vectors produced by the reference's own code that pin it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libalbba_ref.so"
NPARAM = 1443


def build() -> Path:
    subprocess.run(["make", "-s", "-f", str(HERE / "Makefile")], check=True)
    return LIB


def reference_root() -> Path | None:
    """The reference source tree used by the checker builds: the environment
    variable ALB_REFERENCE_ROOT, else the default of oracle/Makefile.ref;
    None when no reference tree is there (e.g. on a machine that only runs
    the prebuilt checker)."""
    root = os.environ.get("ALB_REFERENCE_ROOT")
    if not root:
        r = subprocess.run(["make", "-s", "-f", str(HERE / "Makefile.ref"), "print-ref"],
                           capture_output=True, text=True)
        root = r.stdout.strip() if r.returncode == 0 else ""
    if root and Path(root, "bfs", "src", "bfs_ref.h").exists():
        return Path(root)
    return None


def build_reference(ref_root: str | os.PathLike | None = None) -> Path | None:
    """Compile the reference's own sources + harness into oracle/_ref (if present)."""
    root = Path(ref_root) if ref_root else reference_root()
    if root is None or not Path(root, "bfs", "src", "bfs_ref.h").exists():
        return None
    subprocess.run(["make", "-s", "-f", str(HERE / "Makefile.ref"), f"REF={root}"], check=True)
    return REF_LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.orc_bfs.restype = C.c_int32
        L.orc_bfs.argtypes = [C.c_int64, P, P, P, P, C.c_int32, P, P]
        L.orc_spmv.restype = None
        L.orc_spmv.argtypes = [C.c_int64, P, P, P, P, P]
        L.orc_level_counts.restype = None
        L.orc_level_counts.argtypes = [C.c_int64, P, C.c_int32, P]
        L.orc_validate.restype = C.c_int32
        L.orc_validate.argtypes = [C.c_int64, P, P, P, P, C.c_int32, P, P]
        L.orc_sell_order.restype = None
        L.orc_sell_order.argtypes = [C.c_int64, P, C.c_int32, P]
        L.orc_sell_size.restype = C.c_int64
        L.orc_sell_size.argtypes = [C.c_int64, P, P, C.c_int32, C.c_int32]
        L.orc_sell_build.restype = None
        L.orc_sell_build.argtypes = [C.c_int64, P, P, P, C.c_int32, C.c_int32, P, P, P, P]
        L.orc_sell_long.restype = C.c_int64
        L.orc_sell_long.argtypes = [C.c_int64, P, P, P, C.c_int32, P, P, P]
        L.orc_refalgo_bfs.restype = C.c_int32
        L.orc_refalgo_bfs.argtypes = [C.c_int64, P, P, C.c_int32, C.c_int32, C.c_int32, P,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_refalgo_prepare.restype = C.c_void_p
        L.orc_refalgo_prepare.argtypes = [C.c_int64, P, P, C.c_int32, C.c_int32,
                                          C.POINTER(C.c_double)]
        L.orc_refalgo_run.restype = C.c_int32
        L.orc_refalgo_run.argtypes = [P, C.c_int32, P, C.POINTER(C.c_double)]
        L.orc_refalgo_free.restype = None
        L.orc_refalgo_free.argtypes = [P]
        L.orc_mlp_forward.restype = None
        L.orc_mlp_forward.argtypes = [P, C.c_int32, P, P]
        L.orc_mlp_loss_grad.restype = C.c_float
        L.orc_mlp_loss_grad.argtypes = [P, C.c_int32, P, P, P, P]
        L.orc_adam_step.restype = None
        L.orc_adam_step.argtypes = [P, P, P, P, C.c_int32, C.c_float, C.c_float, C.c_float,
                                    C.c_float]
        _lib = L
    return _lib


def _a(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


def bfs(rowptr, col, root, in_rowptr=None, in_col=None):
    """Levels and min-index parents (symmetric graph when in_* is None)."""
    rp, cl = _a(rowptr, np.int64), _a(col, np.int32)
    irp = rp if in_rowptr is None else _a(in_rowptr, np.int64)
    icl = cl if in_col is None else _a(in_col, np.int32)
    n = rp.shape[0] - 1
    level = np.empty(n, np.int32)
    parent = np.empty(n, np.int32)
    nl = lib().orc_bfs(n, rp.ctypes.data, cl.ctypes.data, irp.ctypes.data, icl.ctypes.data,
                       int(root), level.ctypes.data, parent.ctypes.data)
    return level, parent, nl


def spmv(rowptr, col, val, x):
    """y = A x in fp64, one fused multiply-add per entry in CSR order."""
    rp, cl = _a(rowptr, np.int64), _a(col, np.int32)
    v, xx = _a(val, np.float64), _a(x, np.float64)
    n = rp.shape[0] - 1
    y = np.empty(n, np.float64)
    lib().orc_spmv(n, rp.ctypes.data, cl.ctypes.data, v.ctypes.data, xx.ctypes.data, y.ctypes.data)
    return y


def level_counts(level, num_levels):
    lv = _a(level, np.int32)
    out = np.zeros(max(num_levels, 1), np.int64)
    lib().orc_level_counts(lv.shape[0], lv.ctypes.data, num_levels, out.ctypes.data)
    return out[:num_levels]


def validate(rowptr, col, root, level, parent, in_rowptr=None, in_col=None) -> int:
    rp, cl = _a(rowptr, np.int64), _a(col, np.int32)
    irp = rp if in_rowptr is None else _a(in_rowptr, np.int64)
    icl = cl if in_col is None else _a(in_col, np.int32)
    lv, pa = _a(level, np.int32), _a(parent, np.int32)
    return lib().orc_validate(rp.shape[0] - 1, rp.ctypes.data, cl.ctypes.data, irp.ctypes.data,
                              icl.ctypes.data, int(root), lv.ctypes.data, pa.ctypes.data)


def sell_order(deg, sigma):
    d = _a(deg, np.int32)
    out = np.empty(d.shape[0], np.int32)
    lib().orc_sell_order(d.shape[0], d.ctypes.data, int(sigma), out.ctypes.data)
    return out


def sell_build(rowptr, col, order, C_, long_row=0):
    """Position-space SELL layout; rows longer than long_row (> 0) stay empty."""
    rp, cl, od = _a(rowptr, np.int64), _a(col, np.int32), _a(order, np.int32)
    n = rp.shape[0] - 1
    ns = (n + C_ - 1) // C_
    size = lib().orc_sell_size(n, rp.ctypes.data, od.ctypes.data, C_, int(long_row))
    inv = np.empty(n, np.int32)
    width = np.empty(ns, np.int32)
    off = np.empty(ns + 1, np.int64)
    scol = np.empty(max(size, 1), np.int32)
    lib().orc_sell_build(n, rp.ctypes.data, cl.ctypes.data, od.ctypes.data, C_, int(long_row),
                         inv.ctypes.data, width.ctypes.data, off.ctypes.data, scol.ctypes.data)
    return inv, width, off, scol[:size]


def sell_long(rowptr, col, order, long_row):
    """(lrow, lptr, lcol) of the rows longer than long_row, position space."""
    rp, cl, od = _a(rowptr, np.int64), _a(col, np.int32), _a(order, np.int32)
    n = rp.shape[0] - 1
    k = lib().orc_sell_long(n, rp.ctypes.data, cl.ctypes.data, od.ctypes.data, int(long_row),
                            None, None, None)
    lrow = np.empty(max(k, 1), np.int32)
    lptr = np.empty(k + 1, np.int64)
    lib().orc_sell_long(n, rp.ctypes.data, cl.ctypes.data, od.ctypes.data, int(long_row),
                        lrow.ctypes.data, lptr.ctypes.data, None)
    lcol = np.empty(max(int(lptr[-1]), 1), np.int32)
    lib().orc_sell_long(n, rp.ctypes.data, cl.ctypes.data, od.ctypes.data, int(long_row),
                        lrow.ctypes.data, lptr.ctypes.data, lcol.ctypes.data)
    return lrow[:k], lptr, lcol[: int(lptr[-1])]


def refalgo_bfs(rowptr, col, root, sigma=16384, ntasks=0):
    """The reference's level loop restated on the CPU: (counts, bfs_ms, conv_ms)."""
    rp, cl = _a(rowptr, np.int64), _a(col, np.int32)
    n = rp.shape[0] - 1
    counts = np.zeros(n + 1, np.int64)
    bms, cms = C.c_double(), C.c_double()
    nl = lib().orc_refalgo_bfs(n, rp.ctypes.data, cl.ctypes.data, int(root), int(sigma),
                               int(ntasks), counts.ctypes.data, C.byref(bms), C.byref(cms))
    return counts[:nl], bms.value, cms.value


class RefAlgo:
    """The reference's level loop restated on the CPU, SELL built once."""

    def __init__(self, rowptr, col, sigma=16384, ntasks=0):
        self._rp, self._col = _a(rowptr, np.int64), _a(col, np.int32)
        self.n = self._rp.shape[0] - 1
        cms = C.c_double()
        self._h = lib().orc_refalgo_prepare(self.n, self._rp.ctypes.data, self._col.ctypes.data,
                                            int(sigma), int(ntasks), C.byref(cms))
        self.conv_ms = cms.value

    def run(self, root):
        counts = np.zeros(self.n + 1, np.int64)
        bms = C.c_double()
        nl = lib().orc_refalgo_run(self._h, int(root), counts.ctypes.data, C.byref(bms))
        return counts[:nl], bms.value

    def close(self):
        if self._h:
            lib().orc_refalgo_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


def mlp_forward(params, x):
    p, xx = _a(params, np.float32), _a(x, np.float32)
    b = xx.shape[0]
    out = np.empty((b, 3), np.float32)
    lib().orc_mlp_forward(p.ctypes.data, b, xx.ctypes.data, out.ctypes.data)
    return out


def mlp_loss_grad(params, x, y, mask):
    p, xx, yy, mm = (_a(params, np.float32), _a(x, np.float32), _a(y, np.float32),
                     _a(mask, np.float32))
    g = np.empty(NPARAM, np.float32)
    loss = lib().orc_mlp_loss_grad(p.ctypes.data, xx.shape[0], xx.ctypes.data, yy.ctypes.data,
                                   mm.ctypes.data, g.ctypes.data)
    return float(loss), g


def adam_step(params, grad, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """In place on params, m, v (float32 arrays)."""
    lib().orc_adam_step(params.ctypes.data, _a(grad, np.float32).ctypes.data, m.ctypes.data,
                        v.ctypes.data, int(t), lr, b1, b2, eps)


# ------------------------------------------------ the reference's own code
_ref = None


def ref_lib() -> C.CDLL | None:
    """oracle/_ref/libalbba_ref.so built from the reference sources (None if absent)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            return None
        L = C.CDLL(str(REF_LIB))
        P = C.c_void_p
        L.refh_bfs_counts.restype = C.c_int
        L.refh_bfs_counts.argtypes = [C.c_int, P, P, P]
        L.refh_sell.restype = C.c_int
        L.refh_sell.argtypes = [C.c_int, P, P, C.c_int, C.c_int, P, P, P, P]
        L.refh_sell_dfc.restype = C.c_int
        L.refh_sell_dfc.argtypes = [C.c_int, P, P, C.c_int, P, P]
        L.refh_custom_bfs.restype = C.c_int
        L.refh_custom_bfs.argtypes = [C.c_int, P, P, C.c_int, P, P, P]
        _ref = L
    return _ref

"""Generate tests/golden/mtx/*.mtx and tests/golden/mtx.json from the
reference's own Matrix Market reader and undirected conversion.

The .mtx files are small seeded inputs written here (general, symmetric,
hermitian, skew-symmetric; pattern, real, integer, complex; entries in no
particular order, with repeats, self-loops, comment and blank lines). For
each, the record holds the CSR that the reference's reader builds
(mmio_info + mmio_data, bfs/src/mmio_highlevel.h:11-263) and, for files that
are not symmetric, the undirected graph of the reference driver
(bfs/src/main.c:127-163: convert_csr_to_csc + MergeArr, utils.c:351-380),
both through oracle/_ref/libalbba_ref.so (oracle/ref/ref_harness.c).

Run:  python tests/golden/make_golden_mtx.py   (needs the reference tree)
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
MTX = OUT / "mtx"

# name, rows, entries, type, symmetry, seed
SPECS = [
    ("general_pattern", 60, 240, "pattern", "general", 1),
    ("general_real", 45, 200, "real", "general", 2),
    ("general_integer_repeats", 30, 150, "integer", "general", 3),
    ("symmetric_real", 50, 160, "real", "symmetric", 4),
    ("symmetric_pattern_diag", 40, 120, "pattern", "symmetric", 5),
    ("hermitian_complex", 35, 100, "complex", "hermitian", 6),
    ("skew_integer", 30, 90, "integer", "skew-symmetric", 7),
    ("general_complex", 25, 80, "complex", "general", 8),
    ("empty", 5, 0, "pattern", "general", 9),
]


def write_mtx(path: Path, n: int, m: int, typ: str, sym: str, seed: int) -> None:
    rng = np.random.default_rng(seed)
    i = rng.integers(0, n, m)
    j = rng.integers(0, n, m)
    if sym in ("symmetric", "hermitian"):  # one triangle, diagonal allowed
        i, j = np.maximum(i, j), np.minimum(i, j)
    elif sym == "skew-symmetric":  # strictly lower
        keep = i != j
        i, j = np.maximum(i[keep], j[keep]), np.minimum(i[keep], j[keep])
        m = i.shape[0]
    lines = [f"%%MatrixMarket Matrix Coordinate {typ.upper() if seed % 2 else typ} {sym}",
             "% written by tests/golden/make_golden_mtx.py", "%", ""]
    lines.append(f"{n} {n} {m}")
    for a, b in zip(i, j):
        if typ == "pattern":
            lines.append(f"{a + 1} {b + 1}")
        elif typ == "integer":
            lines.append(f"{a + 1} {b + 1} {int(rng.integers(-9, 10))}")
        elif typ == "real":
            lines.append(f"{a + 1}  {b + 1}  {rng.normal():.6e}")
        else:
            lines.append(f"{a + 1} {b + 1} {rng.normal():.4f} {rng.normal():.4f}")
    path.write_text("\n".join(lines) + "\n")


def main() -> None:
    oracle.build_reference()
    L = oracle.ref_lib()
    if L is None:
        raise SystemExit("reference tree not found")
    P = C.c_void_p
    L.refh_mtx_info.restype = C.c_int
    L.refh_mtx_info.argtypes = [C.c_char_p, P, P, P, P]
    L.refh_mtx_data.restype = C.c_int
    L.refh_mtx_data.argtypes = [C.c_char_p, C.c_int, C.c_int, P, P]
    L.refh_undirected.restype = C.c_int
    L.refh_undirected.argtypes = [C.c_int, P, P, P, P]
    MTX.mkdir(exist_ok=True)
    recs = []
    for name, n, m, typ, sym, seed in SPECS:
        path = MTX / f"{name}.mtx"
        write_mtx(path, n, m, typ, sym, seed)
        info = np.zeros(4, np.int32)
        rc = L.refh_mtx_info(str(path).encode(), info[0:].ctypes.data, info[1:].ctypes.data,
                             info[2:].ctypes.data, info[3:].ctypes.data)
        assert rc == 0, (name, rc)
        rows, cols, nnz, issym = (int(x) for x in info)
        rp = np.zeros(rows + 1, np.int32)
        col = np.zeros(max(nnz, 1), np.int32)
        assert L.refh_mtx_data(str(path).encode(), rows, nnz, rp.ctypes.data, col.ctypes.data) == 0
        rec = {"name": name, "file": f"mtx/{name}.mtx", "n": rows, "symmetric": issym,
               "rowptr": rp.tolist(), "col": col[:nnz].tolist()}
        if not issym:
            urp = np.zeros(rows + 1, np.int32)
            ucol = np.zeros(max(2 * nnz, 1), np.int32)
            k = L.refh_undirected(rows, rp.ctypes.data, col.ctypes.data, urp.ctypes.data,
                                  ucol.ctypes.data)
            rec["undirected_rowptr"] = urp.tolist()
            rec["undirected_col"] = ucol[:k].tolist()
        recs.append(rec)
    (OUT / "mtx.json").write_text(json.dumps(recs, separators=(",", ":")))
    print(f"wrote {len(recs)} records")


if __name__ == "__main__":
    main()

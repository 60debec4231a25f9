"""Generate tests/golden/spmv.json from the reference's own fp64 SpMV.

For each case of spmv_cases.py the reference's convert_csr_to_sellcs_dfc
(bfs/src/sparse_matrix.c:523-623, C = 256) builds its SELL-C-sigma matrix
and kernel_SELLCS_DFC (bfs/src/bfs_par_kernels.c:8-53, through the scalar
restatement of its VE intrinsics in oracle/ref/ve_scalar.c, fused
multiply-add as the VE's vfmadd) computes y = A x; the record keeps the
SHA-256 of y's bytes and its first entries as exact bit patterns.

Run:  python tests/golden/make_golden_spmv.py   (needs the reference tree)
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE))

import oracle  # noqa: E402
from spmv_cases import CASES, GOLDEN, digest, inputs  # noqa: E402


def main() -> None:
    if oracle.build_reference() is None:
        sys.exit("reference tree not found")
    R = oracle.ref_lib()
    R.refh_spmv_dfc.restype = None
    R.refh_spmv_dfc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                C.c_void_p, C.c_void_p]
    recs = []
    for case in CASES:
        n, rp, col, val, x = inputs(case)
        rp32 = rp.astype(np.int32)
        for sigma in (256, 16384):  # the DFC build needs sigma >= C = 256
            y = np.full(n, np.nan)
            R.refh_spmv_dfc(n, rp32.ctypes.data, col.ctypes.data, val.ctypes.data, sigma,
                            x.ctypes.data, y.ctypes.data)
            recs.append({"case": case["name"], "sigma": sigma, "n": n, "nnz": int(rp[-1]),
                         "sha256": digest(y),
                         "head_bits": [f"{v:016x}" for v in y[:16].view(np.uint64)]})
    GOLDEN.write_text(json.dumps(recs, indent=1))
    print(f"{len(recs)} spmv records")


if __name__ == "__main__":
    main()

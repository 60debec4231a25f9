"""In-tree build of the albba_gb300 native library (and the oracle checker).

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host C++ (generators, error
plumbing) is compiled by g++ with OpenMP. Objects go to ``_build/`` and the
shared library to ``albba_gb300/libalbba_gb300.so``. Rebuilds are incremental
by file modification time; translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = ROOT / "_build"
LIB = PKG / "libalbba_gb300.so"
PLUGIN = PKG / "libbfs_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if r.stdout.strip() and os.environ.get("ALB_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout)


CHECKED_LIB = PKG / "libalbba_gb300_checked.so"


def _compile_cmd(src: Path, obj: Path, cuda: Path, defs: tuple[str, ...] = ()) -> list[str]:
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    if src.suffix == ".cu":
        return [str(cuda / "bin" / "nvcc"), *ARCH, "-O3", "-lineinfo", "-std=c++17",
                "-Xcompiler", "-fPIC,-fopenmp,-Wall", "--expt-relaxed-constexpr", *defs,
                *inc, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        return ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall",
                f"-I{cuda / 'include'}", *inc, "-c", str(src), "-o", str(obj)]
    # plain C (the reference-facing plugin shim)
    return ["gcc", "-O2", "-std=c11", "-fPIC", "-Wall", *inc, "-c", str(src), "-o", str(obj)]


def build_library(jobs: int | None = None, checked: bool = False) -> Path:
    """Compile and link libalbba_gb300.so and libbfs_gb300.so; return the former.
    checked=True: the bounds-checked variant libalbba_gb300_checked.so
    (-DALB_CHECKED: every vertex id a traversal kernel loads is checked
    before use and a bad one reported as ALB_ERR_DEVICE), objects apart."""
    cuda = _cuda_home()
    bdir = BUILD / "checked" if checked else BUILD
    bdir.mkdir(parents=True, exist_ok=True)
    lib = CHECKED_LIB if checked else LIB
    defs = ("-DALB_CHECKED",) if checked else ()
    hdrs = _headers()
    srcs = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    plugin_src = CSRC / "bfs_plugin.c"
    todo = []
    objs = []
    for s in srcs + ([plugin_src] if plugin_src.exists() and not checked else []):
        o = bdir / (s.name + ".o")
        if s != plugin_src:
            objs.append(o)
        if _stale(o, [s, *hdrs]):
            todo.append((s, o))
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(lambda so: _run(_compile_cmd(so[0], so[1], cuda, defs)), todo))
    if _stale(lib, objs):
        _run([str(cuda / "bin" / "nvcc"), *ARCH, "-shared", "-o", str(lib), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp"])
    if checked:
        return lib
    if plugin_src.exists():
        pobj = BUILD / (plugin_src.name + ".o")
        if _stale(PLUGIN, [pobj, LIB]):
            _run(["gcc", "-shared", "-o", str(PLUGIN), str(pobj), f"-L{PKG}", "-lalbba_gb300",
                  "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build_library())

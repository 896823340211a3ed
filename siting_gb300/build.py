"""Builds the native parts of siting_gb300 in-tree.

* ``siting_gb300/libsiting_gb300.so``: the C-ABI library (include/siting.h),
  CUDA kernels compiled for sm_103a only.
* ``siting_gb300/cusite``: the command-line drop-in over that library.

Each translation unit is compiled in parallel into ``siting_gb300/_build``;
an object is rebuilt only when its source or a header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsiting_gb300.so")
CLI = os.path.join(PKG, "cusite")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xptxas", "-O3",
              "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-O2",
              "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ...")
    if verbose and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles the library and the CLI; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) +
                     [os.path.join(CSRC, f) for f in ("demgen.cpp", "serve.cpp", "tune.cpp")])
    objs, todo = [], []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
            todo.append([nvcc] + ARCH + NVCC_FLAGS + lang + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda c: _run(c, verbose), todo))
    if todo or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs +
             ["-lcudart", "-lgomp", "-lpthread"], verbose)
    cli_src = os.path.join(CSRC, "cusite.cpp")
    if _stale(CLI, [cli_src, LIB] + headers):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + PKG,
              "-lsiting_gb300", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

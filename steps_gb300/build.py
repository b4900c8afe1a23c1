"""Build recipe of libsteps_gb300.so (sm_103a, in-tree).

Compiles every CUDA translation unit under steps_gb300/csrc with
``nvcc -gencode arch=compute_103a,code=sm_103a`` in parallel and links them
into steps_gb300/_build/libsteps_gb300.so. No cmake, no torch extension
machinery: the library is plain C-ABI (include/steps_gb300.h).
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
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libsteps_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                   "-I", CSRC, "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


# The Ewald table builders decide which lattice terms enter by comparing
# squared distances with the cut exactly as the reference does (separately
# rounded products, no FMA contraction); contracting changes those decisions
# and the cell-centre coordinates (the reference's centre cell is exactly 0).
PER_FILE_FLAGS = {"ewald.cu": ["-fmad=false"]}


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    deps = [src, __file__] + glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "steps_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc_path()] + _flags() + PER_FILE_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc_path()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

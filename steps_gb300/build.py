"""Build recipe of libsteps_gb300.so (sm_103a, in-tree).

Compiles every CUDA translation unit under steps_gb300/csrc with
``nvcc -gencode arch=compute_103a,code=sm_103a`` in parallel and links them
into steps_gb300/_build/libsteps_gb300.so. No cmake, no torch extension
machinery: the library is plain C-ABI (include/steps_gb300.h).

The same sources built with -DSTEPS_CHECK give the debug library
steps_gb300/_build/check/libsteps_gb300_check.so, whose kernels check their
tile, slot, output, table and ordering indices (STEPS_E_BOUNDS).
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
CHECK_DIR = os.path.join(OUT_DIR, "check")
CHECK_LIB = os.path.join(CHECK_DIR, "libsteps_gb300_check.so")
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


def _compile(src: str, out_dir: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(out_dir, os.path.basename(src) + ".o")
    deps = [src, __file__] + glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "steps_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc_path()] + _flags() + extra + PER_FILE_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def _link(objs: list[str], lib: str):
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        cmd = [nvcc_path()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, check: bool = True) -> str:
    """Builds libsteps_gb300.so and, with check=True, the bounds-checked
    libsteps_gb300_check.so; all translation units compile in one pool."""
    variants = [(OUT_DIR, LIB, [])]
    if check:
        variants.append((CHECK_DIR, CHECK_LIB, ["-DSTEPS_CHECK"]))
    for d, _, _ in variants:
        os.makedirs(d, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")), key=os.path.getsize, reverse=True)  # longest first
    jobs = [(s, d, extra) for s in srcs for d, _, extra in variants]
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda j: _compile(j[0], j[1], j[2], verbose), jobs))
    for k, (_, lib, _) in enumerate(variants):
        _link(objs[k::len(variants)], lib)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

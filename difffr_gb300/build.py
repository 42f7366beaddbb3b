"""Builds libdfsph.so in-tree with nvcc for sm_103a (translation units in parallel).

    python -m difffr_gb300.build [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdfsph.so")
# the bounds-checked variant (-DDFSPH_BOUNDS_CHECK): every neighbour index and cell range is
# checked before use and a bad one is reported as a device error (tests only)
LIB_BOUNDS = os.path.join(HERE, "libdfsph_boundscheck.so")
SOURCES = ["abi.cu", "engine_fp32.cu", "engine_fp64.cu", "noalloc.cu", "mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "dfsph.h"))
    return files


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, bounds_check: bool = False) -> str:
    lib = LIB_BOUNDS if bounds_check else LIB
    if not force and up_to_date(lib):
        return lib
    bdir = os.path.join(BUILD, "boundscheck") if bounds_check else BUILD
    os.makedirs(bdir, exist_ok=True)
    cc = nvcc()
    extra = ["-DDFSPH_BOUNDS_CHECK"] if bounds_check else []

    def compile_one(src):
        obj = os.path.join(bdir, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, bounds_check="--bounds-check" in sys.argv))

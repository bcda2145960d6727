"""Build recipe for the in-tree CUDA library ``eq_gb300/libeqfield.so`` (sm_103a).

Plain nvcc, no CMake: each translation unit compiles to an object in parallel, then
one link: ``python -m eq_gb300.build``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libeqfield.so")
OBJDIR = os.path.join(HERE, "_build")
SOURCES = [os.path.join(CSRC, f) for f in ("eqf_batch.cu", "eqf_noalloc.cu", "eqf_server.cu",
                                               "eqf_tune.cu", "eqf_output.cpp")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("eqf_common.cuh", "eqf_kernels.cuh",
                                                   "eqf_cells.cuh", "eqf_refine.cuh",
                                                   "eqf_bicgstab.cuh", "eqf_fused.cuh",
                                                   "eqf_rods.cuh", "eqf_walls.cuh",
                                                   "eqf_balance.cuh")] + \
    [os.path.join(ROOT, "include", h) for h in ("eqfield.h", "eqserve.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in DEPS)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-O2", "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    subprocess.run([nvcc(), ARCH, "-shared", "-o", LIB + ".tmp"] + objs, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)

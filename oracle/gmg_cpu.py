"""ctypes loader of the C/OpenMP multigrid-PCG CPU baseline (oracle/csrc/gmg_cpu.c).

TEST/BENCH INFRASTRUCTURE ONLY: the timed CPU baseline with the GPU's algorithm
(matrix-free geometric multigrid preconditioned CG, FP64, one trap per host thread),
beside the reference's assemble + LU per step (cpu_baseline.reference_rate) and the
LU factor kept across steps (cpu_baseline.factor_once_rate).  build() compiles it with
gcc -fopenmp into oracle/libgmg_cpu.so (git-ignored) on whichever host runs it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "gmg_cpu.c")
LIB = os.path.join(HERE, "libgmg_cpu.so")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O3", "-std=c99", "-fopenmp", "-shared", "-fPIC", "-o",
                        LIB + ".tmp", SRC, "-lm"], check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        dp, lp = C.POINTER(C.c_double), C.POINTER(C.c_longlong)
        lib.gmg_cpu_batch.restype = C.c_longlong
        lib.gmg_cpu_batch.argtypes = [C.c_int, dp, lp, dp, dp, C.c_int, C.c_double, C.c_double,
                                      C.c_int, dp, C.POINTER(C.c_int), lp, dp]
        _lib = lib
    return _lib


def run(traps, steps: int, rtol: float = 1e-10, budget_s: float = 1e9, threads: int = 0,
        fields=None):
    """Steps every trap (single species, point cells) from zero (or from `fields`);
    returns (fields, dof_steps, seconds, threads, cg_iterations, per-trap step seconds)."""
    from oracle import hsld
    lib = load()
    par, offs, F, U = [], [0], [], []
    for k, t in enumerate(traps):
        mesh = hsld.RightMesh(t.W, t.H, t.nx, t.ny)
        F.append(hsld.point_load(mesh, t.cell_xy, t.cell_s, scale=t.dt))
        U.append(np.zeros(t.n_nodes) if fields is None else np.array(fields[k], dtype=np.float64))
        par += [t.nx, t.ny, t.W, t.H, t.D[0], t.dt, t.g[0], t.walls]
        offs.append(offs[-1] + t.n_nodes)
    par = np.asarray(par, dtype=np.float64)
    off = np.asarray(offs[:-1], dtype=np.int64)
    Fa = np.concatenate(F)
    Ua = np.concatenate(U)
    sec, thr, its = C.c_double(), C.c_int(), C.c_longlong()
    dp = C.POINTER(C.c_double)
    tsec = np.zeros(len(traps))
    dofs = lib.gmg_cpu_batch(len(traps), par.ctypes.data_as(dp),
                             off.ctypes.data_as(C.POINTER(C.c_longlong)), Fa.ctypes.data_as(dp),
                             Ua.ctypes.data_as(dp), int(steps), float(rtol), float(budget_s),
                             int(threads), C.byref(sec), C.byref(thr), C.byref(its),
                             tsec.ctypes.data_as(dp))
    out = [Ua[offs[k]:offs[k + 1]].copy() for k in range(len(traps))]
    return out, int(dofs), sec.value, thr.value, its.value, tsec


def rate(traps, idx, steps: int, budget_s: float, threads: int = 0):
    """DOF-steps/s of the multigrid-PCG restatement over the sampled traps on the host
    cores: the threads' summed step throughput (one trap per thread at a time, so a
    large batch keeps every thread busy; each trap's one-time hierarchy excluded)."""
    sub = [traps[i] for i in idx]
    _, dofs, sec, thr, its, tsec = run(sub, steps, budget_s=budget_s, threads=threads)
    per_thread = dofs / max(float(np.sum(tsec)), 1e-9)
    return {"value": per_thread * thr, "unit": "DOF-steps/s", "cores": thr, "kind": "port",
            "sample": f"{len(sub)} traps stratified by size, up to {steps} steps each: "
                      f"matrix-free geometric-multigrid preconditioned CG, FP64, rtol 1e-10, "
                      f"C with OpenMP, one trap per thread; value = threads x summed "
                      f"per-trap step throughput",
            "per_thread": per_thread, "cg_iterations": its, "dof_steps": dofs,
            "wall_s": round(sec, 3)}

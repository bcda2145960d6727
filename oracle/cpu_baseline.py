"""Timed CPU baseline: the reference's algorithm for the field step on host cores.

TEST/BENCH INFRASTRUCTURE ONLY (used by bench.py's CPU legs).  Per trap and step it
does what DOLFIN's LinearVariationalSolver::solve does for eQ's hslD form
(src/fHSL.cpp:104-108): re-assemble the system from the element kernels, apply the
Dirichlet rows, LU-factor and solve (scipy SuperLU, serial), so traps run one per
process in a spawn pool over all host cores.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(args):
    (W, H, nx, ny, D, dt, g, walls, xy, s, steps, budget_s, bc, tensor) = args
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from oracle import channel, hsld
    mesh = hsld.RightMesh(W, H, nx, ny)
    F = hsld.point_load(mesh, xy, s, scale=dt)
    u = np.zeros(mesh.n_nodes)
    chans = None
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        if bc is None:
            t3 = tensor if tensor is not None else (None, None, None)
            o = hsld.HsldOracle(W, H, nx, ny, D, dt, g, walls, D11=t3[0], D22=t3[1], D12=t3[2])
            u = o.step(u, F)
        else:  # walls and channels re-assembled every step, as the reference does
            o = channel.MicrofluidicTrap(W, H, nx, ny, D, dt, g, bc["walls"], bc.get("channel"))
            if chans is not None:
                o.channels = chans
            u = o.step(u, F)
            chans = o.channels
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return mesh.n_nodes * done, time.perf_counter() - t0


def reference_rate(traps, idx, steps_per_trap: int, budget_s: float, timeout_s: float = 600.0):
    """DOF-steps/s of assemble + factor + solve per step over the sampled traps."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    jobs = [(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls, t.cell_xy, t.cell_s,
             steps_per_trap, budget_s, getattr(t, "bc", None), getattr(t, "tensor", None))
            for t in (traps[i] for i in idx)]
    procs = min(cores, len(jobs))
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(processes=procs) as pool:
        res = pool.map_async(_worker, jobs).get(timeout=timeout_s)
    wall = time.perf_counter() - t0
    dofs = sum(r[0] for r in res)
    # pool throughput over the compute span (process start-up excluded)
    span = max(r[1] for r in res)
    return {"value": dofs / max(span, 1e-9), "unit": "DOF-steps/s", "cores": procs,
            "kind": "port",
            "sample": f"{len(jobs)} traps stratified by size "
                      f"({sum(traps[i].n_nodes for i in idx)} nodes), up to {steps_per_trap} "
                      f"step(s) each: re-assemble + LU factor + solve per step (scipy SuperLU), "
                      f"one trap per process",
            "dof_steps": int(dofs), "wall_s": round(wall, 3)}


def _factor_once_worker(args):
    (W, H, nx, ny, D, dt, g, walls, xy, s, steps, budget_s) = args
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from oracle import hsld
    t0 = time.perf_counter()
    o = hsld.HsldOracle(W, H, nx, ny, D, dt, g, walls)  # assemble + LU factor, once
    t_factor = time.perf_counter() - t0
    F = hsld.point_load(o.mesh, xy, s, scale=dt)
    u = np.zeros(o.mesh.n_nodes)
    t1 = time.perf_counter()
    done = 0
    for _ in range(steps):
        u = o.step(u, F)  # right-hand side + triangular solves
        done += 1
        if time.perf_counter() - t1 > budget_s:
            break
    return o.mesh.n_nodes * done, time.perf_counter() - t1, t_factor


def factor_once_rate(traps, idx, steps_per_trap: int, budget_s: float,
                     timeout_s: float = 600.0):
    """DOF-steps/s of the same direct solve with the LU factor kept across steps (the
    system matrix does not change between steps of a trap): per step only the
    right-hand side and the two triangular solves; the one-time assembly + factor is
    reported beside it.  One trap per process, serial SuperLU in each."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    jobs = [(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls, t.cell_xy, t.cell_s,
             steps_per_trap, budget_s) for t in (traps[i] for i in idx)]
    procs = min(cores, len(jobs))
    with mp.get_context("spawn").Pool(processes=procs) as pool:
        res = pool.map_async(_factor_once_worker, jobs).get(timeout=timeout_s)
    dofs = sum(r[0] for r in res)
    span = max(r[1] for r in res)
    return {"value": dofs / max(span, 1e-9), "unit": "DOF-steps/s", "cores": procs,
            "kind": "port",
            "sample": f"{len(jobs)} traps stratified by size, up to {steps_per_trap} steps "
                      f"each after one assembly + LU factor (scipy SuperLU), one trap per "
                      f"process",
            "factor_s_total": round(sum(r[2] for r in res), 3), "dof_steps": int(dofs)}


def _rod_worker(args):
    (col, steps, budget_s) = args
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from oracle import hsld, rods_port
    nl = col.n_layers
    fields = np.zeros((nl, col.ny + 1, col.nx + 1))
    ex = rods_port.Exchanger(fields, col.rods, col.ihsl, col.prod, col.mode, col.npm, col.dt,
                             col.km)
    t0 = time.perf_counter()
    t_ex = 0.0
    done = 0
    for _ in range(steps):
        te = time.perf_counter()
        ex.run()  # the cell loop: footprints, gather, exchange, deposit into u0
        t_ex += time.perf_counter() - te
        for l in range(nl):
            o = hsld.HsldOracle(col.W, col.H, col.nx, col.ny, col.D[l], col.dt, col.g[l],
                                col.walls)
            ex.f[l] = o.step(ex.f[l].ravel()).reshape(ex.f[l].shape)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return col.n_nodes * nl * done, time.perf_counter() - t0, t_ex, done * col.n_cells


def rod_colony_rate(colonies, steps: int, budget_s: float, timeout_s: float = 600.0):
    """DOF-steps/s of the reference's coupled step on host cores: the rod cell loop
    (plain-C restatement) then, per layer, re-assemble + LU factor + solve
    (scipy SuperLU), one colony per process."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    jobs = [(c, steps, budget_s) for c in colonies[:max(1, cores)]]
    procs = min(cores, len(jobs))
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(processes=procs) as pool:
        res = pool.map_async(_rod_worker, jobs).get(timeout=timeout_s)
    wall = time.perf_counter() - t0
    dofs = sum(r[0] for r in res)
    span = max(r[1] for r in res)
    t_ex = sum(r[2] for r in res)
    cell_steps = sum(r[3] for r in res)
    return {"value": dofs / max(span, 1e-9), "unit": "DOF-steps/s", "cores": procs,
            "kind": "port",
            "sample": f"{len(jobs)} colonies ({colonies[0].n_cells} rods, {colonies[0].n_layers} "
                      f"layers of {colonies[0].n_nodes} nodes each), up to {steps} step(s) "
                      f"each: rod cell loop in C, then re-assemble + LU factor + solve per "
                      f"layer (scipy SuperLU), one colony per process",
            "exchange_cells_per_s_per_core": cell_steps / max(t_ex, 1e-9),
            "dof_steps": int(dofs), "wall_s": round(wall, 3)}

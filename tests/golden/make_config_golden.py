"""Generates the full-size oracle fixtures of the three solver workloads.

The FP64 oracle (oracle/hsld.py: the hslD assembly of fenics/hslD.h:3103-3533 with the
decay, point-cell and advection extensions, factored once by SuperLU and re-solved
every step) run on the workloads at their stated sizes and step counts:

* single_large_oracle.npz -- 100x40 um, 1024x512 squares (525,825 nodes), 20,000
  cells (seed 1), dt 0.05, 500 steps: per-cell concentrations after every 50 steps,
  nodal fields after steps 50, 250 and 500.
* two_species_oracle.npz -- the same mesh with the advective sender/receiver pair
  (seed 2), 300 steps: per-cell concentrations of both species after every 50 steps,
  both nodal fields after step 300.
* batched_sample_oracle.npz -- the eight traps of the 512-trap uneven batch (seed 3)
  stratified by node count (workloads.stratified_sample), 200 steps each: per-cell
  concentrations after every 50 steps and the nodal field after step 200.

Run from the repository root (about five minutes on eight cores):
    python tests/golden/make_config_golden.py
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

C1_CELLS = tuple(range(50, 501, 50))
C1_NODAL = (50, 250, 500)
C2_CELLS = tuple(range(50, 301, 50))
C3_CELLS = (50, 100, 150, 200)
C3_SEED, C3_TRAPS, C3_SAMPLE = 3, 512, 8


def run(trap, steps, cell_steps, nodal_steps):
    """Steps the oracle, keeping cells and nodal fields at the requested steps."""
    from oracle import hsld
    ns = trap.n_species
    vel = None
    if trap.adv_u:
        u_, L_ = trap.adv_u, trap.adv_len
        vel = lambda x, y: (np.zeros_like(x), -u_ * y / L_)  # noqa: E731
    orc = [hsld.HsldOracle(trap.W, trap.H, trap.nx, trap.ny, trap.D[k], trap.dt, trap.g[k],
                           trap.walls, velocity=vel) for k in range(ns)]
    mesh = orc[0].mesh
    nodes, w = hsld.point_weights(mesh, trap.cell_xy)
    u = [np.zeros(mesh.n_nodes) for _ in range(ns)]
    if ns == 1:
        F = hsld.point_load(mesh, trap.cell_xy, trap.cell_s, scale=trap.dt)
    out = {}
    for n in range(1, steps + 1):
        if ns == 1:
            u[0] = orc[0].step(u[0], F)
        else:  # the explicit sender/receiver coupling of hsld.run_trap
            c1 = np.sum(u[0][nodes] * w, axis=1)
            c2 = np.sum(u[1][nodes] * w, axis=1)
            sig1 = trap.cell_kind * trap.cell_s - 0.05 * c1
            sig2 = (1 - trap.cell_kind) * 0.5 * c1 / (0.1 + c1) - 0.05 * c2
            u = [orc[0].step(u[0], hsld.point_load(mesh, trap.cell_xy, sig1, scale=trap.dt)),
                 orc[1].step(u[1], hsld.point_load(mesh, trap.cell_xy, sig2, scale=trap.dt))]
        if n in cell_steps:
            for k in range(ns):
                out[f"c{k}_{n}"] = np.sum(u[k][nodes] * w, axis=1)
        if n in nodal_steps:
            for k in range(ns):
                out[f"u{k}_{n}"] = u[k].copy()
    return out


def task(name):
    from eq_gb300 import workloads as wl
    t0 = time.time()
    if name == "c1":
        res = run(wl.single_large(1), 500, C1_CELLS, C1_NODAL)
    elif name == "c2":
        res = run(wl.two_species(2), 300, C2_CELLS, (300,))
    else:
        traps = wl.batched_uneven(C3_SEED, C3_TRAPS)
        i = int(name[2:])
        res = run(traps[i], 200, C3_CELLS, (200,))
        res = {f"t{i}_{k}": v for k, v in res.items()}
    print(f"{name}: {time.time() - t0:.0f} s", flush=True)
    return name, res


def main():
    from eq_gb300 import workloads as wl
    sample = wl.stratified_sample(wl.batched_uneven(C3_SEED, C3_TRAPS), C3_SAMPLE)
    names = ["c2", "c1"] + [f"c3{i}" for i in sample]
    with mp.get_context("spawn").Pool(min(len(names), os.cpu_count() or 1)) as pool:
        results = dict(pool.map(task, names))
    np.savez_compressed(os.path.join(HERE, "single_large_oracle.npz"),
                        cell_steps=np.array(C1_CELLS), nodal_steps=np.array(C1_NODAL),
                        **results["c1"])
    np.savez_compressed(os.path.join(HERE, "two_species_oracle.npz"),
                        cell_steps=np.array(C2_CELLS), **results["c2"])
    c3 = {}
    for i in sample:
        c3.update(results[f"c3{i}"])
    np.savez_compressed(os.path.join(HERE, "batched_sample_oracle.npz"),
                        traps=np.array(sample), seed=C3_SEED, n_traps=C3_TRAPS,
                        cell_steps=np.array(C3_CELLS), **c3)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()

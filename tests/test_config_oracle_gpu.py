"""The solver workloads at their stated sizes and step counts against the FP64 oracle's
committed fixtures (tests/golden/make_config_golden.py), through the C ABI:

* the 100x40 um trap of 1024x512 squares (525,825 nodes, 20,000 cells), 500 steps:
  per-cell concentrations after every 50 steps, nodal fields after 50, 250, 500;
* the same mesh with the advective sender/receiver species pair, 300 steps;
* the eight traps of the 512-trap uneven batch stratified by size, 200 steps, in one
  batch.

Tolerances (relative L2): 1e-9 for the plain FP64 form, 1e-6 for the chosen
FP32 + FP64-refinement form.  Every step's FP64 mass balance is kept on and its drift
checked at the solver tolerance."""
import os

import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {F.FP64: 1e-9, F.FP32_IR: 1e-6}
DRIFT = {F.FP64: 1e-9, F.FP32_IR: 3e-7}  # FP32 form: ten times its default rtol (3e-8)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def tparams(t, k=0):
    return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[k], t.dt, t.g[k], t.walls, adv_u=t.adv_u,
                         adv_len=t.adv_len)


def load(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_single_large_trap_full_size_against_oracle(lib, precision):
    g = load("single_large_oracle.npz")
    t = wl.single_large(1)
    worst = 0.0
    with F.TrapBatch([tparams(t)], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.mass_balance(True)
        done = 0
        for n in g["cell_steps"]:
            b.step(int(n) - done)
            done = int(n)
            e = rel(b.read_cells(0), g[f"c0_{n}"])
            worst = max(worst, e)
            assert e <= TOL[precision], (n, e)
            if n in g["nodal_steps"]:
                e = rel(b.read_nodal(0), g[f"u0_{n}"])
                assert e <= TOL[precision], (n, e)
        bal = b.read_balance(0)
    assert done == 500 and bal["steps"] == 500
    assert bal["drift_rel_max"] <= DRIFT[precision], bal
    print(f"precision {precision}: worst cells relL2 {worst:.3e}, "
          f"drift_rel_max {bal['drift_rel_max']:.3e}")


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_two_species_full_size_against_oracle(lib, precision):
    g = load("two_species_oracle.npz")
    t = wl.two_species(2)
    with F.TrapBatch([tparams(t, 0), tparams(t, 1)], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.couple_species(0, 1, t.cell_kind, vmax=0.5, K=0.1, uptake=0.05)
        b.mass_balance(True)
        done = 0
        for n in g["cell_steps"]:
            b.step(int(n) - done)
            done = int(n)
            for k in range(2):
                e = rel(b.read_cells(k), g[f"c{k}_{n}"])
                assert e <= TOL[precision], (k, n, e)
        for k in range(2):
            assert rel(b.read_nodal(k), g[f"u{k}_300"]) <= TOL[precision], k
            assert b.read_balance(k)["drift_rel_max"] <= DRIFT[precision], k
    assert done == 300


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_batched_sample_full_steps_against_oracle(lib, precision):
    g = load("batched_sample_oracle.npz")
    traps = wl.batched_uneven(int(g["seed"]), int(g["n_traps"]))
    idx = [int(i) for i in g["traps"]]
    assert idx == wl.stratified_sample(traps, len(idx))
    sub = [traps[i] for i in idx]
    with F.TrapBatch([tparams(t) for t in sub], F.default_opts(precision)) as b:
        for k, t in enumerate(sub):
            b.set_cells(k, t.cell_xy, t.cell_s)
        b.mass_balance(True)
        done = 0
        for n in g["cell_steps"]:
            b.step(int(n) - done)
            done = int(n)
            for k, i in enumerate(idx):
                e = rel(b.read_cells(k), g[f"t{i}_c0_{n}"])
                assert e <= TOL[precision], (i, n, e)
        for k, i in enumerate(idx):
            assert rel(b.read_nodal(k), g[f"t{i}_u0_200"]) <= TOL[precision], i
            assert b.read_balance(k)["drift_rel_max"] <= DRIFT[precision], i
    assert done == 200

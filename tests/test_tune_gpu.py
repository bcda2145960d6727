"""The autotuner (eqf_autotune / eqf_create_tuned) on the GPU."""
import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import hsld

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def tp(t):
    return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)


def test_autotune_table_and_tuned_batch(lib):
    traps = [wl.single_small(0), wl.scaled(wl.single_large(1), 512, 256, n_cells=800)]
    opts = F.default_opts(F.FP32_IR)
    table = F.autotune([tp(t) for t in traps], opts, budget_s=8.0)
    rows = F.tune_table_dict(table)
    assert [r["max_nodes"] for r in rows][:3] == [32768, 131072, 524288]
    used = {0, 2}  # 13,041 and 131,841 nodes
    for k, r in enumerate(rows):
        if k in used:
            assert r["dof_steps_per_s"] > 0
            assert r["tile_nodes"] in (0, 2048, 8192)
            assert 1 <= r["cheb_pre"] <= 3 and 1 <= r["cheb_post"] <= 3
        else:
            assert r["dof_steps_per_s"] == 0
    refs = [hsld.run_trap(t, steps=6) for t in traps]
    with F.TrapBatch([tp(t) for t in traps], opts, tune=table) as b:
        for i, t in enumerate(traps):
            b.set_cells(i, t.cell_xy, t.cell_s)
        b.step(6)
        for i in range(2):
            assert rel(b.read_nodal(i), refs[i]["u"][0]) <= 1e-6
            assert rel(b.read_cells(i), refs[i]["cells"][0]) <= 1e-6

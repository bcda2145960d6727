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
            assert r["tile_nodes"] in (0, 2048, 6144)
            assert r["tile_cols"] in (0, 64, 256, 512)
            assert 1 <= r["cheb_pre"] <= 3 and 1 <= r["cheb_post"] <= 3
            assert (r["max_iters"], r["max_sweeps"]) in ((opts.max_iters, opts.max_sweeps),
                                                        (2, 4), (3, 3))
        else:
            assert r["dof_steps_per_s"] == 0
    # every measured candidate is logged; the chosen configuration is a logged one with
    # the rate the table reports (the Krylov schedules compete in longer trials of their
    # own, so the chosen rate need not be the highest short-trial rate)
    log = table.log
    assert log and {int(c["bucket"]) for c in log} == used
    keys = ("tile_nodes", "tile_cols", "cheb_pre", "cheb_post", "max_iters", "max_sweeps")
    for k in used:
        match = [c for c in log if int(c["bucket"]) == k and
                 all(int(c[f]) == rows[k][f] for f in keys) and
                 c["dof_steps_per_s"] == pytest.approx(rows[k]["dof_steps_per_s"], rel=1e-6)]
        assert match, (k, rows[k])
    refs = [hsld.run_trap(t, steps=6) for t in traps]
    with F.TrapBatch([tp(t) for t in traps], opts, tune=table) as b:
        for i, t in enumerate(traps):
            b.set_cells(i, t.cell_xy, t.cell_s)
        b.step(6)
        for i in range(2):
            assert rel(b.read_nodal(i), refs[i]["u"][0]) <= 1e-6
            assert rel(b.read_cells(i), refs[i]["cells"][0]) <= 1e-6


@pytest.mark.parametrize("cols", [16, 64, 256, 512])
def test_fused_tile_widths_solve_the_same_system(lib, cols):
    """The fused level kernels on 2-D tiles of other widths (eqf_solver_opts.tile_cols):
    the same solution within the chosen form's tolerance, on traps narrower and wider
    than the tiles."""
    traps = wl.batched_uneven(3, 512)
    sub = [traps[i] for i in (int(np.argmin([t.n_nodes for t in traps])), 17, 301)]
    refs = [hsld.run_trap(t, steps=8) for t in sub]
    with F.TrapBatch([tp(t) for t in sub], F.default_opts(F.FP32_IR, tile_cols=cols,
                                                          use_graph=1)) as b:
        for i, t in enumerate(sub):
            b.set_cells(i, t.cell_xy, t.cell_s)
        b.step(8)
        for i in range(len(sub)):
            assert rel(b.read_nodal(i), refs[i]["u"][0]) <= 1e-6
            assert rel(b.read_cells(i), refs[i]["cells"][0]) <= 1e-6


def test_tile_width_is_checked(lib):
    from eq_gb300._lib import EqfError
    t = wl.single_small(0)
    for bad in (8, 30, 1024):
        with pytest.raises(EqfError):
            F.TrapBatch([tp(t)], F.default_opts(F.FP32_IR, tile_cols=bad))

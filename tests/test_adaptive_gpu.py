"""Adaptive refinement sweeps inside the step's CUDA graph (a conditional WHILE node)
against the same sweeps added from the host, through the C ABI.

The graph form runs the same kernels in the same order as the host loop, so the
fields are bit-identical and the per-trap sweep and iteration counts agree; a trap
that still misses rtol after the added sweeps is reported by the next eqf_sync
instead of by eqf_step (which no longer waits for the step)."""
import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def tp(t):
    return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)


def _run(traps, opts, steps):
    with F.TrapBatch([tp(t) for t in traps], opts) as b:
        for i, t in enumerate(traps):
            b.set_cells(i, t.cell_xy, t.cell_s)
        b.step(steps)
        b.sync()
        u = [b.read_nodal(i) for i in range(len(traps))]
        st = [b.stats(i) for i in range(len(traps))]
    return u, st


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_graph_loop_is_bit_identical_to_host_loop(lib, precision):
    traps = wl.batched_uneven(3, 512)
    sub = [traps[i] for i in (int(np.argmin([t.n_nodes for t in traps])), 17, 301, 402)]
    # a tight rtol with one scheduled sweep makes steps need added sweeps
    kw = dict(adaptive=1, max_sweeps=1, rtol=1e-10 if precision == F.FP32_IR else 1e-12)
    ug, sg = _run(sub, F.default_opts(precision, use_graph=1, **kw), 10)
    uh, sh = _run(sub, F.default_opts(precision, use_graph=0, **kw), 10)
    assert any(s["sweeps"] > s["steps"] for s in sh), "no step needed an added sweep"
    for a, b in zip(ug, uh):
        assert np.array_equal(a, b)
    for a, b in zip(sg, sh):
        assert (a["steps"], a["sweeps"], a["iters"]) == (b["steps"], b["sweeps"], b["iters"])


def test_unconverged_step_is_reported_by_the_next_sync(lib):
    t = wl.single_small(0)
    o = F.default_opts(F.FP64, use_graph=1, adaptive=1, max_sweeps=1, rtol=1e-30)
    with F.TrapBatch([tp(t)], o) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.step(1)  # queues the step and returns
        with pytest.raises(_lib.EqfError) as e:
            b.sync()
        assert e.value.code == _lib.EQF_ERR_NOT_CONVERGED
        st = b.stats(0)
        assert st["steps"] == 1 and st["sweeps"] == 1 + 8
        b.sync()  # reported once
        b.step(2)
        with pytest.raises(_lib.EqfError) as e:
            b.sync()
        assert "2 trap-step" in str(e.value)
    # the host loop reports the same step from eqf_step itself
    o0 = F.default_opts(F.FP64, use_graph=0, adaptive=1, max_sweeps=1, rtol=1e-30)
    with F.TrapBatch([tp(t)], o0) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        with pytest.raises(_lib.EqfError) as e:
            b.step(1)
        assert e.value.code == _lib.EQF_ERR_NOT_CONVERGED

"""Slot reuse (eqf_replace_trap / eqf_replace_traps) through the C ABI.

A trap put into the slot of another gives the same bits as the same trap in a batch
of its own, and the traps around it keep giving the bits they give without the
replacement.  The traps share h = 0.25 um and D, so every batch here has the same
multigrid depth (as a serving cohort's class guarantees)."""
import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def trap(nx, ny, seed, two=False):
    rng = np.random.default_rng(seed)
    W, H = 0.25 * nx, 0.25 * ny
    m = max(4, nx * ny // 50)
    xy = np.stack([rng.uniform(0.1, W - 0.1, m), rng.uniform(0.1, H - 0.1, m)], axis=1)
    if two:
        return wl.Trap(W=W, H=H, nx=nx, ny=ny, D=[490.0, 300.0], g=[0.01, 0.02], dt=0.1,
                       steps=1, cell_xy=xy, cell_s=np.ones(m),
                       cell_kind=(rng.uniform(size=m) < 0.5).astype(np.int32),
                       adv_u=0.5, adv_len=40.0)
    return wl.Trap(W=W, H=H, nx=nx, ny=ny, D=[490.0], g=[0.01], dt=0.1, steps=1,
                   cell_xy=xy, cell_s=rng.lognormal(0.0, 0.5, m))


def params(t):
    return [F.trap_params(t.W, t.H, t.nx, t.ny, t.D[k], t.dt, t.g[k], t.walls,
                          adv_u=t.adv_u, adv_len=t.adv_len) for k in range(len(t.D))]


def load(b, slot, t):
    b.set_cells(slot, t.cell_xy, t.cell_s)
    if len(t.D) == 2:  # species 2 takes the same cells
        b.couple_species(slot, slot + 1, t.cell_kind)


def alone(t, steps):
    tp = params(t)
    with F.TrapBatch(tp, F.default_opts(F.FP32_IR, use_graph=1)) as b:
        load(b, 0, t)
        b.step(steps)
        return [b.read_nodal(k) for k in range(len(tp))], [b.read_cells(k) for k in range(len(tp))]


def test_replaced_slot_gives_the_bits_of_a_fresh_batch(lib):
    A, B, C, D = trap(200, 96, 1), trap(160, 80, 2), trap(48, 40, 3), trap(150, 64, 4)
    with F.TrapBatch(params(A) + params(B) + params(C), F.default_opts(F.FP32_IR, use_graph=1)) as b:
        for slot, t in enumerate((A, B, C)):
            load(b, slot, t)
        b.step(5)
        b.set_active(1, False)  # B finished: frozen, then reused
        b.step(1)
        b.replace_trap(1, params(D)[0])
        assert b.num_nodes(1) == D.n_nodes  # the new geometry is in place at once
        load(b, 1, D)
        b.step(7)
        got_d = (b.read_nodal(1), b.read_cells(1))
        got_a = b.read_nodal(0)
        got_c = b.read_nodal(2)
    ud, cd = alone(D, 7)
    assert np.array_equal(got_d[0], ud[0]) and np.array_equal(got_d[1], cd[0])
    assert np.array_equal(got_a, alone(A, 13)[0][0])
    assert np.array_equal(got_c, alone(C, 13)[0][0])


def test_replaced_advective_pair(lib):
    P1, P2, P3 = trap(96, 48, 11, two=True), trap(80, 40, 12, two=True), trap(72, 36, 13, two=True)
    with F.TrapBatch(params(P1) + params(P2), F.default_opts(F.FP32_IR, use_graph=1)) as b:
        load(b, 0, P1)
        load(b, 2, P2)
        b.step(4)
        b.set_active(2, False)
        b.set_active(3, False)
        b.replace_traps([2, 3], params(P3))  # both species in one call (one rebuild)
        load(b, 2, P3)
        b.step(5)
        got3 = [b.read_cells(2), b.read_cells(3)]
        got1 = [b.read_cells(0), b.read_cells(1)]
    _, c3 = alone(P3, 5)
    _, c1 = alone(P1, 9)
    for g, a in zip(got3 + got1, c3 + c1):
        assert np.array_equal(g, a)


def test_replacement_must_fit_its_slot(lib):
    A, B = trap(120, 60, 21), trap(64, 32, 22)
    with F.TrapBatch(params(A) + params(B), F.default_opts(F.FP32_IR, use_graph=1)) as b:
        load(b, 0, A)
        load(b, 1, B)
        b.step(2)
        # wider or taller than slot 1; and 60 x 24, smaller, whose 3-cell rows at level 3
        # are not halved again where the slot's 4-cell rows are: larger at levels 4, 5
        for bad in (trap(72, 32, 23), trap(64, 40, 24), trap(60, 24, 26)):
            assert not b.slot_fits(1, params(bad)[0])
            with pytest.raises(_lib.EqfError) as e:
                b.replace_trap(1, params(bad)[0])
            assert e.value.code == _lib.EQF_ERR_INVALID
        assert b.slot_fits(1, params(trap(60, 30, 27))[0])
        adv = trap(32, 16, 25, two=True)
        with pytest.raises(_lib.EqfError):  # advective trap into a CG batch
            b.replace_trap(1, params(adv)[0])
        b.step(3)  # untouched by the refused calls
        got = b.read_nodal(0)
    assert np.array_equal(got, alone(A, 5)[0][0])

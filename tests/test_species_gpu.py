"""Two coupled species with advection (the sender/receiver layer pair) and the
BiCGSTAB inner solve, through the C ABI, against the FP64 oracle."""
import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import hsld

pytestmark = pytest.mark.gpu
TOL = {F.FP64: 1e-9, F.FP32_IR: 1e-6}  # relL2 of the plain and the chosen form


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def species_params(t):
    return [F.trap_params(t.W, t.H, t.nx, t.ny, t.D[k], t.dt, t.g[k], t.walls, adv_u=t.adv_u,
                          adv_len=t.adv_len) for k in range(t.n_species)]


def run_pair(t, steps, precision, **opts):
    with F.TrapBatch(species_params(t), F.default_opts(precision, **opts)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.couple_species(0, 1, t.cell_kind, vmax=0.5, K=0.1, uptake=0.05)
        b.step(steps)
        return ([b.read_nodal(0), b.read_nodal(1)], [b.read_cells(0), b.read_cells(1)],
                [b.stats(0), b.stats(1)])


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_two_species_with_advection_against_oracle(lib, precision):
    t = wl.scaled(wl.two_species(2), 128, 64, n_cells=400)
    steps = 12
    ref = hsld.run_trap(t, steps=steps)
    u, c, _ = run_pair(t, steps, precision, use_graph=1)
    for k in range(2):
        assert rel(u[k], ref["u"][k]) <= TOL[precision], k
        assert rel(c[k], ref["cells"][k]) <= TOL[precision], k
    # the receivers' species is produced only through the coupling
    assert np.linalg.norm(ref["u"][1]) > 0


def test_two_species_graph_and_eager_agree_bitwise(lib):
    t = wl.scaled(wl.two_species(2), 96, 48, n_cells=200)
    a = run_pair(t, 6, F.FP32_IR, use_graph=1)
    b = run_pair(t, 6, F.FP32_IR, use_graph=0)
    for k in range(2):
        assert np.array_equal(a[0][k], b[0][k])
        assert np.array_equal(a[1][k], b[1][k])


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_bicgstab_on_the_symmetric_operator(lib, precision):
    t = wl.single_small(0)
    ref = hsld.run_trap(t, steps=10)
    tp = F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)
    with F.TrapBatch([tp], F.default_opts(precision, krylov=F.KRYLOV_BICGSTAB)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.step(10)
        assert rel(b.read_nodal(0), ref["u"][0]) <= TOL[precision]
        assert rel(b.read_cells(0), ref["cells"][0]) <= TOL[precision]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_single_species_advection_strong_flow(lib, precision):
    """A flow 200x the colony outflow (cell Peclet ~0.02): the operator is clearly
    nonsymmetric, the automatic choice is BiCGSTAB."""
    t = wl.scaled(wl.single_small(0), 160, 80, n_cells=300)
    t.adv_u, t.adv_len = 100.0, 40.0
    ref = hsld.run_trap(t, steps=8)
    tp = F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls, adv_u=t.adv_u,
                       adv_len=t.adv_len)
    with F.TrapBatch([tp], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.step(8)
        assert rel(b.read_nodal(0), ref["u"][0]) <= TOL[precision]
        assert rel(b.read_cells(0), ref["cells"][0]) <= TOL[precision]


def test_coupled_pair_in_a_batch_is_bit_identical_to_alone(lib):
    """Batched with another pair of the same multigrid depth the pair is bit-identical
    to the pair alone; batched with a trap that needs more levels (the hierarchy depth
    is the batch's) it agrees to well within the solver tolerance."""
    t = wl.scaled(wl.two_species(2), 96, 48, n_cells=200)
    alone = run_pair(t, 5, F.FP32_IR, use_graph=1)
    u = wl.scaled(wl.two_species(2), 96, 48, n_cells=150, seed=9)
    tps = species_params(u) + species_params(t)
    with F.TrapBatch(tps, F.default_opts(F.FP32_IR, use_graph=1)) as b:
        b.set_cells(0, u.cell_xy, u.cell_s)
        b.couple_species(0, 1, u.cell_kind, vmax=0.5, K=0.1, uptake=0.05)
        b.set_cells(2, t.cell_xy, t.cell_s)
        b.couple_species(2, 3, t.cell_kind, vmax=0.5, K=0.1, uptake=0.05)
        b.step(5)
        for k in range(2):
            assert np.array_equal(b.read_nodal(2 + k), alone[0][k])
            assert np.array_equal(b.read_cells(2 + k), alone[1][k])
    other = wl.single_small(0)
    tps = [F.trap_params(other.W, other.H, other.nx, other.ny, other.D[0], other.dt,
                         other.g[0], other.walls)] + species_params(t)
    with F.TrapBatch(tps, F.default_opts(F.FP32_IR, use_graph=1)) as b:
        b.set_cells(0, other.cell_xy, other.cell_s)
        b.set_cells(1, t.cell_xy, t.cell_s)
        b.couple_species(1, 2, t.cell_kind, vmax=0.5, K=0.1, uptake=0.05)
        b.step(5)
        for k in range(2):
            assert rel(b.read_nodal(1 + k), alone[0][k]) <= 10 * b.opts.rtol

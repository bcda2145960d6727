"""GPU solver behaviour through the C ABI: fixtures, determinism, batching, the
reference's step semantics and full-size properties."""
import os

import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import hsld

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {F.FP64: 1e-9, F.FP32_IR: 1e-6}  # relL2 targets of the plain and the chosen form


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def tparams(t):
    return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
@pytest.mark.parametrize("graph", [0, 1])
def test_single_small_fixture_100_steps(lib, precision, graph):
    d = np.load(os.path.join(GOLDEN, "single_small_oracle.npz"))
    t = wl.single_small(0)
    with F.TrapBatch([tparams(t)], F.default_opts(precision, use_graph=graph)) as b:
        b.set_cells(0, d["xy"], d["s"])
        done = 0
        for n in (1, 10, 100):
            b.step(n - done)
            done = n
            assert rel(b.read_nodal(0), d[f"u_{n}"]) <= TOL[precision]
            assert rel(b.read_cells(0), d[f"c_{n}"]) <= TOL[precision]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_odd_mesh_fixture(lib, precision):
    d = np.load(os.path.join(GOLDEN, "odd_mesh_oracle.npz"))
    for walls in (1, 0, 13):
        tp = F.trap_params(16.5, 3.5, 33, 7, 49.0, 0.1, 0.01, walls)
        with F.TrapBatch([tp], F.default_opts(precision)) as b:
            b.set_cells(0, d["xy"], d["s"])
            b.step(8)
            assert rel(b.read_nodal(0), d[f"u_walls{walls}"]) <= TOL[precision]
            assert rel(b.read_cells(0), d[f"c_walls{walls}"]) <= TOL[precision]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_trap_in_a_batch_is_bit_identical_to_alone(lib, precision):
    traps = wl.batched_uneven(3, 5)
    o = F.default_opts(precision, use_graph=1)
    alone = []
    for t in traps[:2]:
        with F.TrapBatch([tparams(t)], o) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            b.step(6)
            alone.append((b.read_nodal(0), b.read_cells(0)))
    # the same two traps, in another order and mixed with others
    order = [4, 1, 3, 0, 2]
    with F.TrapBatch([tparams(traps[i]) for i in order], o) as b:
        for k, i in enumerate(order):
            b.set_cells(k, traps[i].cell_xy, traps[i].cell_s)
        b.step(6)
        for i in (0, 1):
            k = order.index(i)
            assert np.array_equal(b.read_nodal(k), alone[i][0])
            assert np.array_equal(b.read_cells(k), alone[i][1])


def test_deposit_is_bit_identical_under_cell_permutation(lib):
    t = wl.single_small(0)
    rng = np.random.default_rng(4)
    xy = np.concatenate([t.cell_xy, t.cell_xy[:20]])  # include coincident cells
    s = np.concatenate([t.cell_s, rng.uniform(0.5, 2.0, 20)])
    perm = rng.permutation(len(s))
    res = []
    for p in (np.arange(len(s)), perm):
        with F.TrapBatch([tparams(t)], F.default_opts(F.FP64)) as b:
            b.set_cells(0, xy[p], s[p])
            b.step(3)
            res.append(b.read_nodal(0))
    assert np.array_equal(res[0], res[1])


def test_rate_update_equals_fresh_cells(lib):
    t = wl.single_small(0)
    s2 = np.linspace(0.1, 3.0, t.n_cells)
    with F.TrapBatch([tparams(t)], F.default_opts(F.FP64)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.set_cell_rates(0, s2)
        b.step(4)
        u1 = b.read_nodal(0)
    with F.TrapBatch([tparams(t)], F.default_opts(F.FP64)) as b:
        b.set_cells(0, t.cell_xy, s2)
        b.step(4)
        u2 = b.read_nodal(0)
    assert np.array_equal(u1, u2)


def test_batch_wide_cell_io_matches_per_trap(lib):
    traps = wl.batched_uneven(3, 3)
    with F.TrapBatch([tparams(t) for t in traps], F.default_opts(F.FP32_IR)) as b:
        for i, t in enumerate(traps):
            b.set_cells(i, t.cell_xy, t.cell_s)
        rates = np.concatenate([t.cell_s * 1.5 for t in traps])
        b.set_cell_rates_all(rates)
        b.step(3)
        allc = b.read_cells_all()
        per = np.concatenate([b.read_cells(i) for i in range(3)])
        assert np.array_equal(allc, per)


def test_batch_wide_rates_survive_a_cell_rebuild(lib):
    """Batch-wide rates live on the device until a rebuild needs them: replacing one
    trap's cells afterwards keeps the other traps' batch-wide rates."""
    traps = wl.batched_uneven(4, 3)
    new = [t.cell_s * (2.0 + i) for i, t in enumerate(traps)]
    moved = wl.batched_uneven(5, 3)[1]
    res = []
    for via_all in (True, False):
        with F.TrapBatch([tparams(t) for t in traps], F.default_opts(F.FP64)) as b:
            for i, t in enumerate(traps):
                b.set_cells(i, t.cell_xy, t.cell_s)
            b.step(1)
            if via_all:
                b.set_cell_rates_all(np.concatenate(new))
            else:
                for i in range(3):
                    b.set_cell_rates(i, new[i])
            xy = np.clip(moved.cell_xy, 0, [traps[1].W, traps[1].H])
            b.set_cells(1, xy, moved.cell_s)  # rebuild: traps 0 and 2 keep `new`
            b.step(2)
            res.append(np.concatenate([b.read_nodal(i) for i in range(3)]))
    assert np.array_equal(res[0], res[1])


def test_reference_step_semantics_through_the_mirror(lib):
    """FieldSolver: deposits added into solution_vector, then stepDiffusion (as the
    reference's controller/worker exchange does), against the oracle."""
    p = F.DiffusionParams(dt=0.1, D_HSL=490.0, trapWidthMicrons=40.0, trapHeightMicrons=20.0,
                          nodesPerMicron=2.0)
    fs = F.FieldSolver("THREEWALLED")
    fs.initDiffusion(p)
    o = hsld.HsldOracle(40.0, 20.0, 80, 40, 490.0, 0.1, 0.0, walls=1)
    u = np.zeros(o.mesh.n_nodes)
    rng = np.random.default_rng(8)
    for step in range(6):
        nodes = rng.integers(81 * 2, o.mesh.n_nodes, 12)
        inc = rng.uniform(0.0, 1.0, 12)
        np.add.at(fs.solution_vector, nodes, inc)
        np.add.at(u, nodes, inc)
        fs.stepDiffusion()
        u = o.step(u)
        assert rel(fs.solution_vector, u) <= 1e-9
        assert abs(fs.getBoundaryFlux()["totalFlux"] - o.boundary_flux(u)) <= \
            1e-9 * abs(o.boundary_flux(u))
    fs.finalize()


def test_add_nodal_equals_adding_on_the_host(lib):
    t = wl.single_small(0)
    nodes = np.array([500, 501, 500, 7000, 12000, 7000])
    inc = np.array([1.0, 0.25, 0.5, 2.0, 0.1, 0.3])
    with F.TrapBatch([tparams(t)], F.default_opts(F.FP64)) as b:
        b.add_nodal(0, nodes, inc)
        u = b.read_nodal(0)
    ref = np.zeros(t.n_nodes)
    np.add.at(ref, nodes, inc)
    assert np.allclose(u, ref, rtol=0, atol=1e-15)


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_mass_is_conserved_with_zero_flux_walls(lib, precision):
    tp = F.trap_params(20.0, 10.0, 80, 40, 490.0, 0.1, 0.0, 0)
    rng = np.random.default_rng(2)
    u0 = rng.uniform(0.0, 1.0, 81 * 41)
    with F.TrapBatch([tp], F.default_opts(precision)) as b:
        b.set_nodal(0, u0)
        m0 = b.total_mass(0)
        b.step(20)
        m1 = b.total_mass(0)
    # each step conserves 1^T M u up to the solve tolerance (rtol |b| per step)
    rtol = F.default_opts(precision).rtol
    assert abs(m1 - m0) <= (2e-9 if precision == F.FP64 else 20 * rtol) * m0


def test_large_trap_scaled_copy_against_oracle(lib):
    t = wl.scaled(wl.single_large(1), 256, 128, n_cells=2000)
    ref = hsld.run_trap(t, steps=30)
    for precision in (F.FP64, F.FP32_IR):
        with F.TrapBatch([tparams(t)], F.default_opts(precision, use_graph=1)) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            b.step(30)
            assert rel(b.read_nodal(0), ref["u"][0]) <= TOL[precision]
            assert rel(b.read_cells(0), ref["cells"][0]) <= TOL[precision]


def test_large_trap_full_size_chosen_form_against_plain_form(lib):
    """Size-independent property at 1024x512 squares (525,825 nodes): the chosen form
    stays within relL2 1e-6 of the plain FP64 form over 150 steps, and both conserve
    the mass balance identically."""
    t = wl.single_large(1)
    out = {}
    for precision in (F.FP64, F.FP32_IR):
        with F.TrapBatch([tparams(t)], F.default_opts(precision, use_graph=1)) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            snaps = []
            for _ in range(3):
                b.step(50)
                snaps.append((b.read_nodal(0), b.read_cells(0), b.total_mass(0)))
            out[precision] = snaps
    for (u64, c64, m64), (u32, c32, m32) in zip(out[F.FP64], out[F.FP32_IR]):
        assert rel(u32, u64) <= 1e-6 and rel(c32, c64) <= 1e-6
        assert abs(m32 - m64) <= 1e-6 * m64


def test_batched_sample_against_oracle(lib):
    traps = wl.batched_uneven(3, 512)
    idx = [int(np.argmin([t.n_nodes for t in traps])), 17, 301]
    sub = [traps[i] for i in idx]
    refs = [hsld.run_trap(t, steps=12) for t in sub]
    with F.TrapBatch([tparams(t) for t in sub], F.default_opts(F.FP32_IR, use_graph=1)) as b:
        for k, t in enumerate(sub):
            b.set_cells(k, t.cell_xy, t.cell_s)
        b.step(12)
        for k in range(len(sub)):
            assert rel(b.read_nodal(k), refs[k]["u"][0]) <= 1e-6
            assert rel(b.read_cells(k), refs[k]["cells"][0]) <= 1e-6


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_fused_and_unfused_level_kernels_agree(lib, precision):
    """The one-kernel bottom levels, the temporally blocked level kernels (default)
    and the step-by-step kernels solve the same systems: all meet the oracle's
    tolerance and agree closely."""
    t = wl.scaled(wl.single_large(1), 256, 128, n_cells=2000)
    ref = hsld.run_trap(t, steps=12)
    out = []
    for fuse in (2, 1, 0):
        with F.TrapBatch([tparams(t)], F.default_opts(precision, use_graph=1,
                                                      fuse_levels=fuse)) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            b.step(12)
            u = b.read_nodal(0)
            assert rel(u, ref["u"][0]) <= TOL[precision]
            out.append(u)
    assert rel(out[0], out[2]) <= TOL[precision]
    assert rel(out[1], out[2]) <= TOL[precision]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_cg_update_folded_into_finest_level_kernel(lib, precision):
    """With the fused finest level, each CG iteration's x += alpha p, r -= alpha q runs
    inside the next iteration's k_down (and the last one inside the refinement update):
    no k_cg_update launch, the same iteration counts, the oracle's answer.  The
    step-by-step V-cycle keeps the separate update kernel."""
    t = wl.scaled(wl.single_large(1), 256, 128, n_cells=2000)
    ref = hsld.run_trap(t, steps=6)
    prof, stats = {}, {}
    for fuse in (1, 0):
        with F.TrapBatch([tparams(t)], F.default_opts(precision, use_graph=0,
                                                      fuse_levels=fuse)) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            b.step(5)
            b.profile(True)
            b.step(1)
            b.sync()
            prof[fuse] = b.profile_read()
            b.profile(False)
            assert rel(b.read_nodal(0), ref["u"][0]) <= TOL[precision]
            assert rel(b.read_cells(0), ref["cells"][0]) <= TOL[precision]
            stats[fuse] = b.stats(0)
    assert prof[1]["cg_update"]["launches"] == 0 and prof[1]["down0_cg"]["launches"] > 0
    assert prof[0]["cg_update"]["launches"] > 0 and prof[0]["down0_cg"]["launches"] == 0
    # one count per Krylov iteration in both: at most max_iters a sweep
    mi = F.default_opts(precision).max_iters
    for f in (1, 0):
        assert 0 < stats[f]["iters"] <= mi * stats[f]["sweeps"]


def coarse_launches(b):
    """Launches of the coarse-level class in one profiled step: the one-kernel bottom
    levels replace several launches per V-cycle, so fewer launches show that it ran."""
    b.profile(True)
    b.step(1)
    b.sync()
    n = b.profile_read()["coarse"]["launches"]
    b.profile(False)
    return n


def test_bottom_levels_kernel_on_uneven_traps(lib):
    """Uneven traps of a batch share the level count; the one-kernel bottom levels
    (per trap, in shared memory) give the step-by-step path's solution."""
    traps = wl.batched_uneven(6, 6)
    res, launches = [], []
    for fuse in (2, 0):
        with F.TrapBatch([tparams(t) for t in traps],
                         F.default_opts(F.FP32_IR, use_graph=1, fuse_levels=fuse)) as b:
            for i, t in enumerate(traps):
                b.set_cells(i, t.cell_xy, t.cell_s)
            b.step(5)
            res.append([b.read_nodal(i) for i in range(len(traps))])
            launches.append(coarse_launches(b))
    for a, c in zip(res[0], res[1]):
        assert rel(a, c) <= 1e-6
    assert launches[0] < launches[1]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_bottom_levels_kernel_is_bit_identical_to_level_kernels(lib, precision):
    """The one-kernel bottom levels evaluate the fused level kernels' expressions on
    the same operands: the same bits whichever level the batch starts it at."""
    traps = wl.batched_uneven(3, 4)
    res, launches = [], []
    for fuse in (2, 1):
        with F.TrapBatch([tparams(t) for t in traps],
                         F.default_opts(precision, use_graph=1, fuse_levels=fuse)) as b:
            for i, t in enumerate(traps):
                b.set_cells(i, t.cell_xy, t.cell_s)
            b.step(4)
            res.append([b.read_nodal(i) for i in range(len(traps))])
            launches.append(coarse_launches(b))
    for a, c in zip(res[0], res[1]):
        assert np.array_equal(a, c)
    assert launches[0] < launches[1]  # k_bottom ran

"""Anisotropic per-node diffusion tensors on the GPU (eqf_set_tensor) against the FP64
oracle, whose element tensors are pinned to the reference's generated hslD kernel."""
import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import hsld
from oracle import rods as R

pytestmark = pytest.mark.gpu
TOL = {F.FP64: 1e-9, F.FP32_IR: 1e-6}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def smooth_field(nx, ny, W, H, Dx=2.0, Dy=0.4):
    y, x = np.meshgrid(np.linspace(0, H, ny + 1), np.linspace(0, W, nx + 1), indexing="ij")
    theta = 0.7 * np.sin(2 * np.pi * x / W) + 0.5 * y / H
    return [v.ravel() for v in wl.rotated_tensor(theta, Dx, Dy)]


def run_pair(t, D11, D22, D12, steps, precision, walls=wl.WALL_BOTTOM):
    tp = F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], walls)
    o = hsld.HsldOracle(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], walls, D11=D11, D22=D22,
                        D12=D12)
    Fl = hsld.point_load(o.mesh, t.cell_xy, t.cell_s, scale=t.dt)
    u = np.zeros(o.mesh.n_nodes)
    for _ in range(steps):
        u = o.step(u, Fl)
    with F.TrapBatch([tp], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.set_tensor(0, D11, D22, D12)
        b.step(steps)
        return b.read_nodal(0), u


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_smooth_tensor_field_against_oracle(lib, precision):
    t = wl.scaled(wl.single_small(0), 80, 40, n_cells=80)
    D11, D22, D12 = smooth_field(t.nx, t.ny, t.W, t.H)
    got, ref = run_pair(t, D11, D22, D12, 6, precision)
    assert rel(got, ref) <= TOL[precision]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_rod_oriented_tensor_against_oracle(lib, precision):
    """The reference's tensor: (1, 1, 0) except on each rod's footprint, where the
    rotated diag(Dx, Dy) of the rod's angle is written (later cells win)."""
    col = wl.rod_colony(seed=4, W=20.0, H=10.0, npm=4.0, n_cells=60)
    nx, ny = col.nx, col.ny
    D11, D22, D12 = np.ones((ny + 1, nx + 1)), np.ones((ny + 1, nx + 1)), np.zeros((ny + 1, nx + 1))
    for r in col.rods:
        theta = np.arctan2(r["body_rot"][1], r["body_rot"][0])
        a, b_, c = wl.rotated_tensor(theta, 5.0, 0.5)
        for (i, j) in R.footprint(r, col.npm, nx, ny):
            D11[i, j], D22[i, j], D12[i, j] = a, b_, c
    t = wl.scaled(wl.single_small(0), nx, ny, n_cells=50)
    t.W, t.H = col.W, col.H
    t.cell_xy = np.stack([np.random.default_rng(1).uniform(0.5, col.W - 0.5, 50),
                          np.random.default_rng(2).uniform(0.5, col.H - 0.5, 50)], 1)
    got, ref = run_pair(t, D11.ravel(), D22.ravel(), D12.ravel(), 5, precision,
                        walls=wl.WALL_BOTTOM | wl.WALL_TOP)
    assert rel(got, ref) <= TOL[precision]


def test_isotropic_tensor_restores_the_plain_operator_bitwise(lib):
    t = wl.scaled(wl.single_small(0), 64, 32, n_cells=40)
    tp = F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)
    out = []
    for mode in (0, 1):
        with F.TrapBatch([tp], F.default_opts(F.FP32_IR)) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            if mode:
                n = b.num_nodes(0)
                b.set_tensor(0, np.full(n, 3.0), np.full(n, 3.0), np.zeros(n))
                b.set_tensor(0)  # back to isotropic
            b.step(4)
            out.append(b.read_nodal(0))
    assert np.array_equal(out[0], out[1])


def test_tensor_argument_errors(lib):
    t = wl.scaled(wl.single_small(0), 32, 16, n_cells=10)
    tp = F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)
    with F.TrapBatch([tp], F.default_opts(F.FP64)) as b:
        n = b.num_nodes(0)
        with pytest.raises(F.EqfError):  # not positive definite
            b.set_tensor(0, np.ones(n), np.ones(n), np.full(n, 2.0))
        # all three fields or none
        assert b._lib.eqf_set_tensor(b._h, 0, F._dp(np.ones(n)), None, None) == -1


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_mixed_batch_is_bit_identical_to_each_trap_alone(lib, precision):
    """Class-table and general-path traps run as separate launches of the same level
    kernels: a mixed batch gives every trap the bits it gets alone."""
    base = wl.batched_uneven(7, 4)
    traps = [wl.scaled(t, t.nx // 4 * 2, t.ny // 4 * 2, n_cells=60) for t in base]
    tens = {1: smooth_field(traps[1].nx, traps[1].ny, traps[1].W, traps[1].H),
            3: smooth_field(traps[3].nx, traps[3].ny, traps[3].W, traps[3].H, 0.5, 2.0)}
    o = F.default_opts(precision, use_graph=1)

    def tp(t):
        return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)

    alone = []
    for i, t in enumerate(traps):
        with F.TrapBatch([tp(t)], o) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            if i in tens:
                b.set_tensor(0, *tens[i])
            b.step(4)
            alone.append(b.read_nodal(0))
    with F.TrapBatch([tp(t) for t in traps], o) as b:
        for i, t in enumerate(traps):
            b.set_cells(i, t.cell_xy, t.cell_s)
            if i in tens:
                b.set_tensor(i, *tens[i])
        b.step(4)
        for i in range(len(traps)):
            assert np.array_equal(b.read_nodal(i), alone[i])


def test_bottom_levels_kernel_with_general_path_traps(lib):
    """The one-kernel bottom levels fetch a general-path trap's stencils as the level
    kernels do: fuse_levels 2 and 1 give the same bits on a mixed batch."""
    base = wl.batched_uneven(8, 3)
    traps = [wl.scaled(t, t.nx // 4 * 2, t.ny // 4 * 2, n_cells=60) for t in base]
    tens = {0: smooth_field(traps[0].nx, traps[0].ny, traps[0].W, traps[0].H)}
    res, launches = [], []
    for fuse in (2, 1):
        with F.TrapBatch([F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)
                          for t in traps],
                         F.default_opts(F.FP32_IR, use_graph=1, fuse_levels=fuse)) as b:
            for i, t in enumerate(traps):
                b.set_cells(i, t.cell_xy, t.cell_s)
                if i in tens:
                    b.set_tensor(i, *tens[i])
            b.step(3)
            res.append([b.read_nodal(i) for i in range(len(traps))])
            b.profile(True)
            b.step(1)
            b.sync()
            launches.append(b.profile_read()["coarse"]["launches"])
            b.profile(False)
    for a, c in zip(res[0], res[1]):
        assert np.array_equal(a, c)
    assert launches[0] < launches[1]  # the one-kernel bottom levels ran

"""Wall conditions with values, Robin walls and the flow channels of the
MICROFLUIDIC_TRAP mode on the GPU (eqf_set_boundaries), through the C ABI, against
the FP64 oracle (oracle/channel.py)."""
import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from oracle import channel as chn
from oracle import hsld

pytestmark = pytest.mark.gpu
TOL = {F.FP64: 1e-9, F.FP32_IR: 1e-6}
K = {chn.NEUMANN: _lib.EQF_BC_NEUMANN, chn.DIRICHLET: _lib.EQF_BC_DIRICHLET,
     chn.ROBIN: _lib.EQF_BC_ROBIN, chn.CHANNEL: _lib.EQF_BC_CHANNEL, chn.WELL: _lib.EQF_BC_WELL}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


class Case:
    def __init__(self, W, H, nx, ny, D, dt, g, walls, channel=None, cells=0, seed=0):
        self.W, self.H, self.nx, self.ny, self.D, self.dt, self.g = W, H, nx, ny, D, dt, g
        self.walls, self.channel = walls, channel
        rng = np.random.Generator(np.random.PCG64(seed))
        self.xy = np.stack([rng.uniform(0.5, W - 0.5, cells), rng.uniform(0.5, H - 0.5, cells)], 1)
        self.s = rng.uniform(0.5, 2.0, cells)

    def params(self):
        return F.trap_params(self.W, self.H, self.nx, self.ny, self.D, self.dt, self.g, 0)

    def configure(self, b, t):
        b.set_boundaries(t, {side: (K[k], v, r) for side, (k, v, r) in self.walls.items()},
                         self.channel)
        if len(self.s):
            b.set_cells(t, self.xy, self.s)

    def oracle(self, steps):
        tr = chn.MicrofluidicTrap(self.W, self.H, self.nx, self.ny, self.D, self.dt, self.g,
                                  self.walls, self.channel)
        Fl = hsld.point_load(tr.mesh, self.xy, self.s, scale=self.dt) if len(self.s) else None
        u = np.zeros(tr.mesh.n_nodes)
        for _ in range(steps):
            u = tr.step(u, Fl)
        return u, tr.channels


def microfluidic_case(seed=0, nx=64, ny=32, substeps=6):
    W, H = nx * 0.25, ny * 0.25
    D, v = 490.0, 40.0
    rl, rr = chn.robin_rates(v, D, 10.0, 10.0)
    return Case(W, H, nx, ny, D, 0.1, 0.01,
                {chn.BOTTOM: (chn.CHANNEL, 0.0, 0.0), chn.TOP: (chn.CHANNEL, 0.0, 0.0),
                 chn.LEFT: (chn.ROBIN, 0.0, rl), chn.RIGHT: (chn.ROBIN, 0.0, rr)},
                channel={"velocity": v, "D": D, "rate": (rl, rr), "substeps": substeps,
                         "well_scaling": 10.0 * 25.0 * 0.25},
                cells=int(0.02 * nx * ny), seed=seed)


CASES = {
    "dirichlet_values": lambda: Case(10.0, 5.0, 40, 20, 490.0, 0.1, 0.01,
                                     {chn.BOTTOM: (chn.DIRICHLET, 1.0, 0), chn.TOP: (chn.DIRICHLET, 2.0, 0),
                                      chn.LEFT: (chn.DIRICHLET, 0.5, 0), chn.RIGHT: (chn.DIRICHLET, 3.0, 0)},
                                     cells=20, seed=1),
    "robin_load": lambda: Case(12.0, 6.0, 48, 24, 300.0, 0.1, 0.0,
                               {chn.BOTTOM: (chn.DIRICHLET, 0.0, 0), chn.LEFT: (chn.ROBIN, 1.2, 5.0),
                                chn.RIGHT: (chn.ROBIN, 0.3, 20.0), chn.TOP: (chn.ROBIN, 0.0, 2.0)},
                               cells=30, seed=2),
    "microfluidic": microfluidic_case,
}


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
@pytest.mark.parametrize("name", list(CASES))
def test_walls_against_oracle(lib, name, precision):
    c = CASES[name]()
    steps = 6
    u_ref, ch_ref = c.oracle(steps)
    with F.TrapBatch([c.params()], F.default_opts(precision)) as b:
        c.configure(b, 0)
        b.step(steps)
        u = b.read_nodal(0)
        if ch_ref:
            bot, top = b.read_channels(0)
    assert rel(u, u_ref) <= TOL[precision]
    if ch_ref:
        assert rel(bot, ch_ref[chn.BOTTOM]) <= TOL[precision]
        assert rel(top, ch_ref[chn.TOP]) <= TOL[precision]
        assert np.linalg.norm(ch_ref[chn.TOP]) > 0


def test_mixed_batch_each_trap_against_its_oracle(lib):
    plain = Case(10.0, 5.0, 40, 20, 490.0, 0.1, 0.01, {chn.BOTTOM: (chn.DIRICHLET, 0.0, 0)},
                 cells=15, seed=3)
    cases = [plain, microfluidic_case(4, 48, 24), CASES["robin_load"](), microfluidic_case(5, 80, 40)]
    steps = 5
    with F.TrapBatch([c.params() for c in cases], F.default_opts(F.FP32_IR)) as b:
        for t, c in enumerate(cases):
            c.configure(b, t)
        b.step(steps)
        for t, c in enumerate(cases):
            u_ref, ch_ref = c.oracle(steps)
            assert rel(b.read_nodal(t), u_ref) <= 1e-6, t
            if ch_ref:
                bot, top = b.read_channels(t)
                assert rel(bot, ch_ref[chn.BOTTOM]) <= 1e-6, t


def test_microfluidic_graph_and_eager_agree_bitwise(lib):
    c = microfluidic_case(6)
    out = []
    for g in (1, 0):
        with F.TrapBatch([c.params()], F.default_opts(F.FP32_IR, use_graph=g)) as b:
            c.configure(b, 0)
            b.step(5)
            out.append((b.read_nodal(0), *b.read_channels(0)))
    for x, y in zip(*out):
        assert np.array_equal(x, y)


def test_channel_values_round_trip_and_drive_the_walls(lib):
    c = microfluidic_case(7, 32, 16)
    with F.TrapBatch([c.params()], F.default_opts(F.FP64)) as b:
        c.configure(b, 0)
        ramp = np.linspace(0.0, 2.0, c.nx + 1)
        b.set_channels(0, bottom=ramp, top=2.0 - ramp)
        bot, top = b.read_channels(0)
        assert np.array_equal(bot, ramp) and np.array_equal(top, 2.0 - ramp)
        b.step(1)
        U = b.read_nodal(0).reshape(c.ny + 1, c.nx + 1)
        # the wall rows reach the channel values to the solver tolerance
        assert np.allclose(U[0], ramp, rtol=0, atol=1e-9)
        assert np.allclose(U[c.ny], 2.0 - ramp, rtol=0, atol=1e-9)


def test_boundary_argument_errors(lib):
    c = microfluidic_case(8, 32, 16)
    with F.TrapBatch([c.params(), F.trap_params(8.0, 6.0, 32, 16, 490.0, 0.1)],
                     F.default_opts(F.FP64)) as b:
        with pytest.raises(F.EqfError):  # a channel on a side wall
            b.set_boundaries(0, {_lib.EQF_SIDE_LEFT: (_lib.EQF_BC_CHANNEL, 0, 0)}, c.channel)
        with pytest.raises(F.EqfError):  # channel walls need a square lattice
            b.set_boundaries(1, {_lib.EQF_SIDE_BOTTOM: (_lib.EQF_BC_CHANNEL, 0, 0)}, c.channel)
        with pytest.raises(F.EqfError):  # no channel on this trap
            b.read_channels(1)


def test_a_small_batch_does_not_shrink_a_large_channel(lib):
    """Kernel attributes are per kernel: a later batch with short channels must not
    cap the shared memory of an earlier one with long channels (2049 nodes)."""
    big = microfluidic_case(9, 2048, 8, substeps=2)
    small = microfluidic_case(10, 32, 16, substeps=2)
    with F.TrapBatch([big.params()], F.default_opts(F.FP64)) as b1:
        big.configure(b1, 0)
        with F.TrapBatch([small.params()], F.default_opts(F.FP64)) as b2:
            small.configure(b2, 0)
            b2.step(1)
        b1.step(2)
        u_ref, ch_ref = big.oracle(2)
        assert rel(b1.read_nodal(0), u_ref) <= 1e-9
        assert rel(b1.read_channels(0)[0], ch_ref[chn.BOTTOM]) <= 1e-9


@pytest.mark.parametrize("drive", [False, True])
def test_boundary_well_against_oracle(lib, drive):
    """The well integrates the boundary flux every step; with DIRICHLET_UPDATE walls
    (EQF_BC_WELL) its concentration is the walls' value in the next step."""
    W, H, nx, ny = 12.0, 6.0, 48, 24
    scale = 2.0 * 10.0 * 15.0 * (W + H)  # 2*10*(15/lengthScaling)*(W+H)
    decay = 100.0 / W
    walls = ({s_: (chn.WELL, 0.0, 0.0) for s_ in range(4)} if drive
             else {chn.BOTTOM: (chn.DIRICHLET, 0.0, 0.0)})
    c = Case(W, H, nx, ny, 490.0, 0.05, 0.0, walls, cells=40, seed=11)
    tr = chn.MicrofluidicTrap(W, H, nx, ny, 490.0, 0.05, 0.0, walls, None, well=(scale, decay))
    Fl = hsld.point_load(tr.mesh, c.xy, c.s, scale=c.dt)
    u = np.zeros(tr.mesh.n_nodes)
    wells = []
    for _ in range(8):
        u = tr.step(u, Fl)
        wells.append(tr.well_c)
    with F.TrapBatch([c.params()], F.default_opts(F.FP64)) as b:
        c.configure(b, 0)
        b.set_well(0, scale, decay)
        got = []
        for _ in range(8):
            b.step(1)
            got.append(b.read_well(0)[0])
        assert rel(b.read_nodal(0), u) <= 1e-9
    assert max(abs(x - y) for x, y in zip(got, wells)) <= 1e-9 * max(abs(x) for x in wells)
    assert max(wells) > 0

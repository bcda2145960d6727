"""Rod cells of the agent-based model coupled on the GPU (eqf_set_rods and the calls
after it), through the C ABI: the exchange bit for bit against the reference's own
code (golden fixture) and the oracle, the dependency waves, and whole steps
(exchange + solve) against the FP64 oracle."""
import os

import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import hsld
from oracle import rods as R

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "rods_reference.npz")
CASES = ("colony", "walls", "grown", "lattice", "stack")
TOL = {F.FP64: 1e-9, F.FP32_IR: 1e-6}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def layer_params(W, H, npm, nl, D=(490.0, 300.0, 200.0), g=(0.01, 0.02, 0.0), dt=0.1):
    nx, ny = int(W * npm), int(H * npm)
    return [F.trap_params(W, H, nx, ny, D[l], dt, g[l], wl.WALL_BOTTOM) for l in range(nl)]


def golden_case(z, name):
    W, H, npm, dt = (float(v) for v in z[f"{name}/geom"])
    rods = z[f"{name}/rods"].copy().view(_lib.rod_dtype()).ravel()
    return W, H, npm, dt, rods


@pytest.mark.parametrize("name", CASES)
def test_exchange_matches_reference_golden_bitwise(lib, name):
    z = np.load(GOLDEN)
    W, H, npm, dt, rods = golden_case(z, name)
    fin = z[f"{name}/fields_in"]
    nl = fin.shape[0]
    with F.TrapBatch(layer_params(W, H, npm, nl), F.default_opts(F.FP64)) as b:
        for l in range(nl):
            b.set_nodal(l, fin[l].ravel())
        b.set_rods(list(range(nl)), rods, z[f"{name}/ihsl_in"], z[f"{name}/prod"],
                   z[f"{name}/mode"], npm, dt, z[f"{name}/km"])
        for p in range(3):
            b.exchange_rods()
            ih, eh, pts = b.read_rods(0)
            assert np.array_equal(eh, z[f"{name}/ehsl_{p}"]), p
            assert np.array_equal(ih, z[f"{name}/ihsl_{p}"]), p
        assert np.array_equal(pts, z[f"{name}/points"])
        for l in range(nl):
            assert np.array_equal(b.read_nodal(l), z[f"{name}/fields_out"][l].ravel()), l


def oracle_waves(rods, npm, nx, ny):
    """Sequential dependency depth: 1 + the deepest earlier cell sharing a node."""
    last = {}
    wave = []
    for r in rods:
        fp = R.footprint(r, npm, nx, ny)
        w = max((last[p] + 1 for p in fp if p in last), default=0)
        for p in fp:
            last[p] = w
        wave.append(w)
    return max(wave) + 1


@pytest.mark.parametrize("name", ["stack", "colony"])
def test_wave_count_is_the_dependency_depth(lib, name):
    z = np.load(GOLDEN)
    W, H, npm, dt, rods = golden_case(z, name)
    nl = z[f"{name}/fields_in"].shape[0]
    nx, ny = int(W * npm), int(H * npm)
    with F.TrapBatch(layer_params(W, H, npm, nl), F.default_opts(F.FP64)) as b:
        b.set_rods(list(range(nl)), rods, z[f"{name}/ihsl_in"], z[f"{name}/prod"],
                   z[f"{name}/mode"], npm, dt, z[f"{name}/km"])
        waves = b.rod_waves()
        assert waves == oracle_waves(rods, npm, nx, ny)
        # the relaxation settles within the chain length plus its final quiet pass
        passes = b.rod_relax_passes()
        assert (passes == 0) if waves == 1 else (2 <= passes <= waves + 1)
    if name == "stack":
        assert oracle_waves(rods, npm, nx, ny) > 5


@pytest.mark.parametrize("npm", [2.0, 4.0])
def test_large_colony_exchange_bitwise_against_oracle(lib, npm):
    col = wl.rod_colony(seed=21, W=60.0, H=30.0, npm=npm, n_cells=600)
    rng = np.random.Generator(np.random.PCG64(3))
    nl = col.n_layers
    fields = [rng.uniform(0, 30, (col.ny + 1, col.nx + 1)) for _ in range(nl)]
    ih = rng.uniform(0, 5000, (col.n_cells, nl))
    with F.TrapBatch(layer_params(col.W, col.H, col.npm, nl), F.default_opts(F.FP64)) as b:
        for l in range(nl):
            b.set_nodal(l, fields[l].ravel())
        b.set_rods([0, 1], col.rods, ih, col.prod, col.mode, col.npm, col.dt, col.km)
        b.exchange_rods()
        gi, ge, gp = b.read_rods(0)
        gu = [b.read_nodal(l) for l in range(nl)]
        waves = b.rod_waves()
    oi, oe, op = R.exchange(fields, col.rods, ih, col.prod, col.mode, col.npm, col.dt, col.km)
    assert np.array_equal(gp, op)
    assert np.array_equal(ge, oe) and np.array_equal(gi, oi)
    for l in range(nl):
        assert np.array_equal(gu[l], fields[l].ravel()), l
    assert waves >= 2  # random placement overlaps some rods


def run_colony_gpu(col, steps, precision, use_graph=1, traps_first=0):
    nl = col.n_layers
    params = [F.trap_params(col.W, col.H, col.nx, col.ny, col.D[l], col.dt, col.g[l],
                            col.walls) for l in range(nl)]
    # optional unrelated traps in front (the rod layers then sit at other offsets)
    extra = [F.trap_params(10.0, 5.0, 20, 10, 490.0, col.dt, 0.01, wl.WALL_BOTTOM)] * traps_first
    with F.TrapBatch(extra + params, F.default_opts(precision, use_graph=use_graph)) as b:
        layers = list(range(traps_first, traps_first + nl))
        b.set_rods(layers, col.rods, col.ihsl, col.prod, col.mode, col.npm, col.dt, col.km)
        b.step(steps)
        ih, eh, pts = b.read_rods(layers[0])
        return [b.read_nodal(t) for t in layers], ih, eh


def run_colony_oracle(col, steps):
    nl = col.n_layers
    ors = [hsld.HsldOracle(col.W, col.H, col.nx, col.ny, col.D[l], col.dt, col.g[l], col.walls)
           for l in range(nl)]
    f = [np.zeros((col.ny + 1, col.nx + 1)) for _ in range(nl)]
    ih = col.ihsl.copy()
    for _ in range(steps):
        ih, eh, _ = R.exchange(f, col.rods, ih, col.prod, col.mode, col.npm, col.dt, col.km)
        f = [ors[l].step(f[l].ravel()).reshape(f[l].shape) for l in range(nl)]
    return [x.ravel() for x in f], ih, eh


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_coupled_steps_against_oracle(lib, precision):
    col = wl.rod_colony(seed=8, W=24.0, H=12.0, npm=2.0, n_cells=60, dt=0.1)
    steps = 8
    ou, oi, oe = run_colony_oracle(col, steps)
    gu, gi, ge = run_colony_gpu(col, steps, precision, traps_first=1)
    for l in range(col.n_layers):
        assert rel(gu[l], ou[l]) <= TOL[precision], l
    assert rel(gi, oi) <= TOL[precision]
    assert rel(ge, oe) <= TOL[precision]
    assert np.linalg.norm(ou[0]) > 0 and np.linalg.norm(oi[:, 0]) > 0


def test_coupled_steps_graph_and_eager_agree_bitwise(lib):
    col = wl.rod_colony(seed=9, W=30.0, H=14.0, npm=2.0, n_cells=120, dt=0.1)
    a = run_colony_gpu(col, 5, F.FP32_IR, use_graph=1)
    b = run_colony_gpu(col, 5, F.FP32_IR, use_graph=0)
    for x, y in zip(a[0], b[0]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_update_rods_moves_cells_and_keeps_state(lib):
    col = wl.rod_colony(seed=10, W=30.0, H=14.0, npm=2.0, n_cells=80, dt=0.1)
    rng = np.random.Generator(np.random.PCG64(4))
    moved = wl.rod_records(rng.uniform(2, col.W - 2, col.n_cells),
                           rng.uniform(2, col.H - 2, col.n_cells),
                           rng.uniform(0, np.pi, col.n_cells),
                           col.rods["length"], col.W, col.H)
    prod2 = col.prod * 0.5
    nl = col.n_layers
    with F.TrapBatch(layer_params(col.W, col.H, col.npm, nl), F.default_opts(F.FP64)) as b:
        b.set_rods([0, 1], col.rods, col.ihsl, col.prod, col.mode, col.npm, col.dt, col.km)
        b.step(2)
        b.update_rods(0, moved, prod2)
        b.step(2)
        gu = [b.read_nodal(l) for l in range(nl)]
        gi, _, gp = b.read_rods(0)
    ors = [hsld.HsldOracle(col.W, col.H, col.nx, col.ny, 490.0 if l == 0 else 300.0, 0.1,
                           (0.01, 0.02)[l], wl.WALL_BOTTOM) for l in range(nl)]
    f = [np.zeros((col.ny + 1, col.nx + 1)) for _ in range(nl)]
    ih = col.ihsl.copy()
    for s in range(4):
        rods, prod = (col.rods, col.prod) if s < 2 else (moved, prod2)
        ih, _, op = R.exchange(f, rods, ih, prod, col.mode, col.npm, col.dt, col.km)
        f = [ors[l].step(f[l].ravel()).reshape(f[l].shape) for l in range(nl)]
    assert np.array_equal(gp, op)
    for l in range(nl):
        assert rel(gu[l], f[l].ravel()) <= 1e-9
    assert rel(gi, ih) <= 1e-9


def test_frozen_layer_skips_the_exchange(lib):
    col = wl.rod_colony(seed=12, W=20.0, H=10.0, npm=2.0, n_cells=30, dt=0.1)
    nl = col.n_layers
    with F.TrapBatch(layer_params(col.W, col.H, col.npm, nl), F.default_opts(F.FP64)) as b:
        ones = np.ones((col.ny + 1) * (col.nx + 1))
        for l in range(nl):
            b.set_nodal(l, ones)
        b.set_rods([0, 1], col.rods, col.ihsl, col.prod, col.mode, col.npm, col.dt, col.km)
        b._lib.eqf_set_active(b._h, 0, 0)
        b.exchange_rods()
        assert np.array_equal(b.read_nodal(0), ones)
        ih, eh, _ = b.read_rods(0)
        assert np.array_equal(ih, col.ihsl) and not eh.any()
        b._lib.eqf_set_active(b._h, 0, 1)
        b.exchange_rods()
        assert not np.array_equal(b.read_nodal(0), ones)


def test_rod_set_replacement_and_removal(lib):
    col = wl.rod_colony(seed=13, W=20.0, H=10.0, npm=2.0, n_cells=30, dt=0.1)
    with F.TrapBatch(layer_params(col.W, col.H, col.npm, 2), F.default_opts(F.FP64)) as b:
        b.set_rods([0, 1], col.rods, col.ihsl, col.prod, col.mode, col.npm, col.dt, col.km)
        b.step(1)
        few = col.rods[:10]
        b.set_rods([0, 1], few, col.ihsl[:10], col.prod[:10], col.mode[:10], col.npm, col.dt,
                   col.km)
        assert b.read_rods(0)[2].shape == (10,)
        b.step(1)
        b.set_rods([0, 1], few[:0], col.ihsl[:0], col.prod[:0], col.mode[:0], col.npm, col.dt,
                   col.km)
        assert b.rod_waves() == 0
        b.step(1)


def test_rod_argument_errors(lib):
    col = wl.rod_colony(seed=14, W=20.0, H=10.0, npm=2.0, n_cells=10, dt=0.1)
    params = layer_params(col.W, col.H, col.npm, 2) + \
        [F.trap_params(col.W, col.H, 30, 15, 490.0, 0.1, 0.0, wl.WALL_BOTTOM)]
    with F.TrapBatch(params, F.default_opts(F.FP64)) as b:
        args = (col.rods, col.ihsl, col.prod, col.mode)
        with pytest.raises(F.EqfError):   # lattice is not npm nodes per micron
            b.set_rods([0, 1], *args, 3.0, col.dt, col.km)
        with pytest.raises(F.EqfError):   # layers on different meshes
            b.set_rods([0, 2], *args, col.npm, col.dt, col.km)
        bad = col.rods.copy()
        bad["pole_a"][3] = [col.W + 1.0, 1.0]
        with pytest.raises(F.EqfError):   # pole outside the trap
            b.set_rods([0, 1], bad, col.ihsl, col.prod, col.mode, col.npm, col.dt, col.km)
        bad = col.rods.copy()
        bad["length"][0] = 0.5
        with pytest.raises(F.EqfError):   # shorter than its width
            b.set_rods([0, 1], bad, col.ihsl, col.prod, col.mode, col.npm, col.dt, col.km)
        b.set_rods([0, 1], *args, col.npm, col.dt, col.km)
        with pytest.raises(F.EqfError):   # a trap in two rod sets
            b.set_rods([1], col.rods, col.ihsl[:, :1], col.prod[:, :1], col.mode[:, :1],
                       col.npm, col.dt, col.km[:1])
        with pytest.raises(F.EqfError):   # count changes need eqf_set_rods
            b.update_rods(0, col.rods[:5])


def test_several_rod_sets_in_one_batch_bitwise(lib):
    """Colonies with different wave counts share each wave launch."""
    cols = [wl.rod_colony(seed=30, W=24.0, H=12.0, npm=2.0, n_cells=40),
            wl.rod_colony(seed=31, W=20.0, H=10.0, npm=4.0, n_cells=150),
            wl.rod_colony(seed=32, W=16.0, H=8.0, npm=2.0, n_cells=5)]
    rng = np.random.Generator(np.random.PCG64(5))
    params, fields, ihs = [], [], []
    for c in cols:
        params += layer_params(c.W, c.H, c.npm, c.n_layers)
        fields.append([rng.uniform(0, 30, (c.ny + 1, c.nx + 1)) for _ in range(c.n_layers)])
        ihs.append(rng.uniform(0, 3000, (c.n_cells, c.n_layers)))
    with F.TrapBatch(params, F.default_opts(F.FP64)) as b:
        t = 0
        for c, f, ih in zip(cols, fields, ihs):
            for l in range(c.n_layers):
                b.set_nodal(t + l, f[l].ravel())
            b.set_rods(list(range(t, t + c.n_layers)), c.rods, ih, c.prod, c.mode, c.npm, c.dt,
                       c.km)
            t += c.n_layers
        waves = [oracle_waves(c.rods, c.npm, c.nx, c.ny) for c in cols]
        assert b.rod_waves() == max(waves) and len(set(waves)) > 1
        for _ in range(2):
            b.exchange_rods()
            for c, f, ih in zip(cols, fields, ihs):
                ih[:], _, _ = R.exchange(f, c.rods, ih, c.prod, c.mode, c.npm, c.dt, c.km)
        t = 0
        for c, f, ih in zip(cols, fields, ihs):
            gi, _, _ = b.read_rods(t)
            assert np.array_equal(gi, ih)
            for l in range(c.n_layers):
                assert np.array_equal(b.read_nodal(t + l), f[l].ravel())
            t += c.n_layers


def test_batch_wide_rod_update_and_read_match_per_set_calls(lib):
    """update_rods_all / read_rods_all: the same bits as one update_rods / read_rods per
    set (sets taken in increasing order of their first layer)."""
    spec = [(24.0, 12.0, 2.0, 40), (20.0, 10.0, 4.0, 150), (16.0, 8.0, 2.0, 5)]
    cols = [wl.rod_colony(seed=40 + k, W=W, H=H, npm=npm, n_cells=n)
            for k, (W, H, npm, n) in enumerate(spec)]
    moved = [wl.rod_colony(seed=50 + k, W=W, H=H, npm=npm, n_cells=n)
             for k, (W, H, npm, n) in enumerate(spec)]
    rng = np.random.Generator(np.random.PCG64(9))
    params, fields = [], []
    for c in cols:
        params += layer_params(c.W, c.H, c.npm, c.n_layers)
        fields.append([rng.uniform(0, 30, (c.ny + 1, c.nx + 1)) for _ in range(c.n_layers)])
    prods = [rng.uniform(0, 5, (c.n_cells, c.n_layers)) for c in cols]
    out = []
    for batch_wide in (False, True):
        with F.TrapBatch(params, F.default_opts(F.FP64)) as b:
            t, firsts = 0, []
            for c, f in zip(cols, fields):
                for l in range(c.n_layers):
                    b.set_nodal(t + l, f[l].ravel())
                b.set_rods(list(range(t, t + c.n_layers)), c.rods, c.ihsl, c.prod, c.mode,
                           c.npm, c.dt, c.km)
                firsts.append(t)
                t += c.n_layers
            b.exchange_rods()
            if batch_wide:
                b.update_rods_all(np.concatenate([m.rods for m in moved]),
                                  np.concatenate([p.ravel() for p in prods]))
            else:
                for t0, m, p in zip(firsts, moved, prods):
                    b.update_rods(t0, m.rods, p)
            b.exchange_rods()
            b.step(2)
            reads = (b.read_rods_all() if batch_wide
                     else [b.read_rods(t0) for t0 in firsts])
            nod = [b.read_nodal(k) for k in range(len(params))]
            out.append((reads, nod, b.rod_waves()))
    (ra, na, wa), (rb, nb, wb) = out
    assert wa == wb
    for x, y in zip(ra, rb):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)
    for u, v in zip(na, nb):
        assert np.array_equal(u, v)


def test_batch_wide_rod_update_rejects_a_bad_set_before_uploading(lib):
    """update_rods_all with a valid first set and an invalid second one (a pole outside
    the trap) fails and leaves both sets as they were: the next exchange gives the bits
    of a batch that never saw the call."""
    spec = [(24.0, 12.0, 2.0, 40), (20.0, 10.0, 2.0, 30)]
    cols = [wl.rod_colony(seed=60 + k, W=W, H=H, npm=npm, n_cells=n)
            for k, (W, H, npm, n) in enumerate(spec)]
    moved = [wl.rod_colony(seed=70 + k, W=W, H=H, npm=npm, n_cells=n)
             for k, (W, H, npm, n) in enumerate(spec)]
    bad = moved[1].rods.copy()
    bad["pole_a"][3, 0] = spec[1][0] + 5.0
    rng = np.random.Generator(np.random.PCG64(4))
    params, fields = [], []
    for c in cols:
        params += layer_params(c.W, c.H, c.npm, c.n_layers)
        fields.append([rng.uniform(0, 30, (c.ny + 1, c.nx + 1)) for _ in range(c.n_layers)])
    out = []
    for attempt in (False, True):
        with F.TrapBatch(params, F.default_opts(F.FP64)) as b:
            t = 0
            for c, f in zip(cols, fields):
                for l in range(c.n_layers):
                    b.set_nodal(t + l, f[l].ravel())
                b.set_rods(list(range(t, t + c.n_layers)), c.rods, c.ihsl, c.prod, c.mode,
                           c.npm, c.dt, c.km)
                t += c.n_layers
            if attempt:
                with pytest.raises(F.EqfError):
                    b.update_rods_all(np.concatenate([moved[0].rods, bad]))
            b.exchange_rods()
            out.append((b.read_rods_all(), [b.read_nodal(k) for k in range(len(params))]))
    for x, y in zip(out[0][0], out[1][0]):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)
    for u, v in zip(out[0][1], out[1][1]):
        assert np.array_equal(u, v)

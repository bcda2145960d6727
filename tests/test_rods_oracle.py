"""The rod-cell coupling oracle (oracle/rods.py) against the reference's own code:
the golden fixture made from the reference sources (tests/golden/make_rods_golden.py),
hand-counted footprints, and the molecule balance of the exchange.  CPU only."""
import math
import os

import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import workloads as wl
from oracle import ref_rods
from oracle import rods as R
from oracle import rods_port

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "rods_reference.npz")
CASES = ("colony", "walls", "grown", "lattice", "stack")


def golden_case(z, name):
    W, H, npm, dt = (float(v) for v in z[f"{name}/geom"])
    rods = z[f"{name}/rods"].copy().view(_lib.rod_dtype()).ravel()
    return W, H, npm, dt, rods


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_golden_bitwise(name):
    z = np.load(GOLDEN)
    W, H, npm, dt, rods = golden_case(z, name)
    f = [x.copy() for x in z[f"{name}/fields_in"]]
    ih = z[f"{name}/ihsl_in"]
    for p in range(3):
        ih, eh, pts = R.exchange(f, rods, ih, z[f"{name}/prod"], z[f"{name}/mode"], npm, dt,
                                 z[f"{name}/km"])
        assert np.array_equal(eh, z[f"{name}/ehsl_{p}"]), p
        assert np.array_equal(ih, z[f"{name}/ihsl_{p}"]), p
    for l, ref in enumerate(z[f"{name}/fields_out"]):
        assert np.array_equal(f[l], ref), l
    assert np.array_equal(pts, z[f"{name}/points"])


def test_golden_cases_cover_the_edge_cases():
    z = np.load(GOLDEN)
    pts = {n: z[f"{n}/points"] for n in CASES}
    assert (pts["walls"] == 1).sum() >= 5          # centre-node fallback taken
    modes = np.concatenate([z[f"{n}/mode"].ravel() for n in CASES])
    assert set(np.unique(modes)) == {R.HELD, R.CIRCUIT, R.INERT}
    # the stacked cells share nodes: the sequential order matters there
    W, H, npm, dt, rods = golden_case(z, "stack")
    fps = [set(R.footprint(r, npm, int(W * npm), int(H * npm))) for r in rods]
    assert sum(len(a & b) > 0 for i, a in enumerate(fps) for b in fps[i + 1:]) > 20


def test_axis_aligned_footprint_by_hand():
    # a 3-um rod along x at (5, 3) on a 2-nodes/um lattice: its first half's box is
    # x in (4, 6), y in (2.5, 3.5) -> strictly inside: x = 4.5, 5, 5.5 at y = 3
    rods = wl.rod_records([5.0], [3.0], [0.0], [3.0], 10.0, 6.0)
    rods["body_rot"] = [1.0, 0.0]
    pts = R.footprint(rods[0], 2.0, 20, 12)
    assert pts == [(6, 9), (6, 10), (6, 11)]
    # at 4 nodes/um: x in {4.25 .. 5.75} (7 columns), y in {2.75, 3, 3.25} (3 rows)
    pts = R.footprint(rods[0], 4.0, 40, 24)
    assert len(pts) == 21 and pts[0] == (11, 17) and pts[-1] == (13, 23)
    # rows ascending, columns ascending within a row (the reference's search order)
    assert pts == sorted(pts)


def test_short_rod_falls_back_to_its_centre_node():
    # box x in (5.075, 5.125): no lattice column (multiples of 0.5) inside
    rods = wl.rod_records([5.1], [3.2], [0.0], [1.05], 10.0, 6.0)
    rods["body_rot"] = [1.0, 0.0]
    assert R.footprint(rods[0], 2.0, 20, 12) == [(6, 10)]  # round(3.2*2), round(5.1*2)
    # turned by 0.3 rad the same rod covers the node (7, 10) = (5.0, 3.5)
    rods = wl.rod_records([5.1], [3.2], [0.3], [1.05], 10.0, 6.0)
    assert R.footprint(rods[0], 2.0, 20, 12) == [(7, 10)]


def test_pole_quirk_and_clamping():
    # Ecoli::updatePoleCenters: pole B sits 0.5 L + W/2 behind the centre, pole A
    # 0.5 L - W/2 ahead; both are clamped to the trap
    rods = wl.rod_records([1.0], [3.0], [0.0], [3.0], 10.0, 6.0)
    assert rods["pole_a"][0].tolist() == [2.0, 3.0]
    assert rods["pole_b"][0].tolist() == [0.0, 3.0]   # 1 - 2 = -1 -> 0


def test_exchange_conserves_molecules():
    """What leaves the cells (dHSL in molecules) arrives on the lattice: the deposit
    per node times the extracellular area per node (ecf / npm^2), summed."""
    col = wl.rod_colony(seed=5, W=20.0, H=10.0, npm=2.0, n_cells=40)
    rng = np.random.Generator(np.random.PCG64(9))
    nl = col.n_layers
    f = [rng.uniform(0, 10, (col.ny + 1, col.nx + 1)) for _ in range(nl)]
    f0 = [x.copy() for x in f]
    ih = rng.uniform(0, 2000, (col.n_cells, nl))
    # one cell at a time, so that each deposit is attributed to its cell
    for c in range(col.n_cells):
        before = [x.copy() for x in f]
        ih1, eh, pts = R.exchange(f, col.rods[c:c + 1], ih[c:c + 1], col.prod[c:c + 1],
                                  col.mode[c:c + 1], col.npm, col.dt, col.km)
        L = float(col.rods[c]["length"])
        ecf = R.extracellular_fraction(L)
        for l in range(nl):
            inm = ih[c, l] * R.nm_per_molecule(L)
            dH = col.dt * col.km[l] * (inm - eh[0, l])
            sent = R.nm_to_molecules(dH, L)
            arrived = float((f[l] - before[l]).sum()) * ecf / (col.npm * col.npm)
            assert math.isclose(arrived, sent, rel_tol=1e-9, abs_tol=1e-9), (c, l)
    assert any(not np.array_equal(a, b) for a, b in zip(f, f0))


@pytest.mark.skipif(not ref_rods.available(), reason="reference sources not present")
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_matches_reference_on_fresh_colonies(seed):
    ref_rods.build_if_available()
    col = wl.rod_colony(seed=100 + seed, W=24.0, H=12.0, npm=(2.0, 4.0, 2.5)[seed],
                        n_cells=50)
    rng = np.random.Generator(np.random.PCG64(seed))
    nl = col.n_layers
    fields = rng.uniform(0, 40, (nl, col.ny + 1, col.nx + 1))
    ih = rng.uniform(0, 1000, (col.n_cells, nl))
    f = [fields[l].copy() for l in range(nl)]
    i1, e1, p1 = R.exchange(f, col.rods, ih, col.prod, col.mode, col.npm, col.dt, col.km)
    f2, i2, e2, p2 = ref_rods.exchange(fields, col.rods, ih, col.prod, col.mode, col.npm, col.dt,
                                       col.km)
    assert np.array_equal(p1, p2)
    assert np.array_equal(e1, e2) and np.array_equal(i1, i2)
    for l in range(nl):
        assert np.array_equal(f[l], f2[l])


@pytest.mark.parametrize("name", CASES)
def test_c_restatement_matches_reference_golden_bitwise(name):
    """The plain-C restatement (the timed CPU baseline) is the same function."""
    z = np.load(GOLDEN)
    W, H, npm, dt, rods = golden_case(z, name)
    ex = rods_port.Exchanger(z[f"{name}/fields_in"], rods, z[f"{name}/ihsl_in"],
                             z[f"{name}/prod"], z[f"{name}/mode"], npm, dt, z[f"{name}/km"])
    for p in range(3):
        ex.run()
        assert np.array_equal(ex.eh, z[f"{name}/ehsl_{p}"]), p
        assert np.array_equal(ex.ih, z[f"{name}/ihsl_{p}"]), p
    assert np.array_equal(ex.f, z[f"{name}/fields_out"])
    assert np.array_equal(ex.pts, z[f"{name}/points"])

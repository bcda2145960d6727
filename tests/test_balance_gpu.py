"""The per-step FP64 mass balance (eqf_mass_balance / eqf_read_balance) through the
C ABI: its terms against the assembled system of the FP64 oracle on the same fields,
and its drift at the solver's tolerance over 120 steps with sources, decay and a
Dirichlet wall (and with advection, Robin walls and wall values)."""
import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import channel as chn
from oracle import hsld

pytestmark = pytest.mark.gpu
TERMS = ("mass", "mass_prev", "load", "decay", "operator_loss", "wall_outflow", "drift")
# the drift is the solver residual summed over the free rows: |sum r| <= sqrt(N) |r|_2,
# so relative to the mass it stays below a few times the step's rtol
DRIFT = {F.FP64: 1e-9, F.FP32_IR: 3e-7}  # FP32 form: ten times its default rtol (3e-8)
# with wall values the Dirichlet rows' right-hand sides (the values themselves, not
# mass-weighted) dominate |b|, and rtol |b| with them
DRIFT_VALUES = {F.FP64: 1e-8, F.FP32_IR: 1e-6}


def tparams(t, k=0):
    return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[k], t.dt, t.g[k], t.walls, adv_u=t.adv_u,
                         adv_len=t.adv_len)


def check_terms(rec, ref, scale):
    for name in TERMS:
        assert abs(rec[name] - ref[name]) <= 1e-11 * scale, (name, rec[name], ref[name])


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_balance_terms_match_the_assembled_system(lib, precision):
    """Sources, decay and the open bottom wall: each term of the device's balance equals
    the oracle's, evaluated from the assembled matrices on the GPU's own fields."""
    t = wl.single_small(0)
    o = hsld.HsldOracle(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)
    Fl = hsld.point_load(o.mesh, t.cell_xy, t.cell_s, scale=t.dt)
    with F.TrapBatch([tparams(t)], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.mass_balance(True)
        b.step(4)
        for _ in range(3):
            u_old = b.read_nodal(0)
            b.step(1)
            u_new = b.read_nodal(0)
            rec = b.read_balance(0)
            ref = o.balance(u_new, u_old, Fl)
            check_terms(rec, ref, max(ref["mass"], ref["load"]))
            assert rec["wall_outflow"] > 0 and rec["decay"] > 0
            assert rec["operator_loss"] == 0.0
        assert rec["steps"] == 7
        assert abs(rec["load_sum"] - 7 * ref["load"]) <= 1e-12 * 7 * ref["load"]


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_balance_drift_stays_at_solver_tolerance(lib, precision):
    """120 steps of the 40x20 um trap (sources, decay, Dirichlet wall): every step's
    drift stays at the solver tolerance, and the wall outflow is the reference's
    facet flux functional up to the discretisation (same sign, within 20 %)."""
    t = wl.single_small(0)
    with F.TrapBatch([tparams(t)], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.mass_balance(True)
        b.step(120)
        rec = b.read_balance(0)
        flux = b.boundary_flux(0)
    assert rec["steps"] == 120
    assert rec["drift_rel_max"] <= DRIFT[precision], rec
    assert abs(rec["drift_sum"]) <= DRIFT[precision] * rec["load_sum"], rec
    assert flux > 0 and abs(rec["wall_outflow"] - flux) <= 0.2 * flux


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_balance_with_advection(lib, precision):
    """The advective sender/receiver pair: the operator term (advective outflow) is the
    assembled one and both species' drift stays at the solver tolerance."""
    t = wl.scaled(wl.two_species(2), 128, 64, n_cells=400)
    vel = lambda x, y: (np.zeros_like(x), -t.adv_u * y / t.adv_len)  # noqa: E731
    with F.TrapBatch([tparams(t, 0), tparams(t, 1)], F.default_opts(precision)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.couple_species(0, 1, t.cell_kind, vmax=0.5, K=0.1, uptake=0.05)
        b.mass_balance(True)
        b.step(20)
        for k in range(2):
            rec = b.read_balance(k)
            assert rec["drift_rel_max"] <= DRIFT[precision], (k, rec)
            assert rec["operator_loss"] != 0.0
        # one more step checked term by term against the assembled system
        u_old = [b.read_nodal(k) for k in range(2)]
        c_old = [b.read_cells(k) for k in range(2)]
        b.step(1)
        for k in range(2):
            o = hsld.HsldOracle(t.W, t.H, t.nx, t.ny, t.D[k], t.dt, t.g[k], t.walls,
                                velocity=vel, factor=False)
            if k == 0:
                sig = t.cell_kind * t.cell_s - 0.05 * c_old[0]
            else:
                sig = (1 - t.cell_kind) * 0.5 * c_old[0] / (0.1 + c_old[0]) - 0.05 * c_old[1]
            Fl = hsld.point_load(o.mesh, t.cell_xy, sig, scale=t.dt)
            ref = o.balance(b.read_nodal(k), u_old[k], Fl)
            rec = b.read_balance(k)
            check_terms(rec, ref, max(abs(ref["mass"]), abs(ref["load"])))


K = {chn.NEUMANN: _lib.EQF_BC_NEUMANN, chn.DIRICHLET: _lib.EQF_BC_DIRICHLET,
     chn.ROBIN: _lib.EQF_BC_ROBIN}


@pytest.mark.parametrize("precision", [F.FP64, F.FP32_IR])
def test_balance_with_wall_values_and_robin_walls(lib, precision):
    """A Dirichlet wall with a value and Robin walls with external concentrations: the
    load holds the Robin loads, the operator term the Robin outflow, and the terms
    match the assembled system (oracle/channel.py's wall decode)."""
    W, H, nx, ny = 12.0, 6.0, 48, 24
    walls = {chn.BOTTOM: (chn.DIRICHLET, 0.4, 0), chn.LEFT: (chn.ROBIN, 1.2, 5.0),
             chn.RIGHT: (chn.ROBIN, 0.3, 20.0), chn.TOP: (chn.ROBIN, 0.0, 2.0)}
    rng = np.random.Generator(np.random.PCG64(5))
    xy = np.stack([rng.uniform(0.5, W - 0.5, 30), rng.uniform(0.5, H - 0.5, 30)], 1)
    s = rng.uniform(0.5, 2.0, 30)
    tr = chn.MicrofluidicTrap(W, H, nx, ny, 300.0, 0.1, 0.01, walls, None)
    Fl = hsld.point_load(tr.mesh, xy, s, scale=0.1)
    tp = F.trap_params(W, H, nx, ny, 300.0, 0.1, 0.01, 0)
    with F.TrapBatch([tp], F.default_opts(precision)) as b:
        b.set_boundaries(0, {side: (K[k], v, r) for side, (k, v, r) in walls.items()})
        b.set_cells(0, xy, s)
        b.mass_balance(True)
        b.step(30)
        rec = b.read_balance(0)
        assert rec["drift_rel_max"] <= DRIFT_VALUES[precision], rec
        u_old = b.read_nodal(0)
        b.step(1)
        ref = tr.trap.balance(b.read_nodal(0), u_old, Fl)
        rec = b.read_balance(0)
    check_terms(rec, ref, max(abs(ref["mass"]), abs(ref["load"])))
    assert rec["operator_loss"] != 0.0


def test_balance_alone_and_in_a_batch_are_bit_identical(lib):
    """Tile partials summed in tile order per trap: a trap's record does not depend on
    the batch around it; a frozen trap's record stands still."""
    traps = wl.batched_uneven(3, 3)
    recs = []
    with F.TrapBatch([tparams(traps[1])], F.default_opts(F.FP32_IR)) as b:
        b.set_cells(0, traps[1].cell_xy, traps[1].cell_s)
        b.mass_balance(True)
        b.step(5)
        recs.append(b.read_balance(0))
    with F.TrapBatch([tparams(t) for t in traps], F.default_opts(F.FP32_IR)) as b:
        for i, t in enumerate(traps):
            b.set_cells(i, t.cell_xy, t.cell_s)
        b.mass_balance(True)
        b.step(5)
        recs.append(b.read_balance(1))
        frozen = b.read_balance(2)
        b.set_active(2, False)
        b.step(2)
        assert b.read_balance(2) == frozen
        assert b.read_balance(1)["steps"] == 7
    assert recs[0] == recs[1]


def test_balance_carries_mass_and_load_and_refreshes_them(lib):
    """Consecutive steps carry the last mass over as the next starting mass and keep the
    load; new rates or a new field are summed afresh."""
    t = wl.single_small(0)
    o = hsld.HsldOracle(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls, factor=False)
    with F.TrapBatch([tparams(t)], F.default_opts(F.FP64)) as b:
        b.set_cells(0, t.cell_xy, t.cell_s)
        b.mass_balance(True)
        b.step(1)
        r1 = b.read_balance(0)
        b.step(1)
        r2 = b.read_balance(0)
        assert r2["mass_prev"] == r1["mass"] and r2["load"] == r1["load"]
        b.set_cell_rates(0, 2.0 * t.cell_s)
        b.step(1)
        r3 = b.read_balance(0)
        assert r3["mass_prev"] == r2["mass"]
        assert abs(r3["load"] - 2.0 * r2["load"]) <= 1e-13 * r3["load"]
        u = np.random.default_rng(3).uniform(0.0, 1.0, t.n_nodes)
        u[o.dir] = 0.0
        b.set_nodal(0, u)
        b.step(1)
        r4 = b.read_balance(0)
        assert abs(r4["mass_prev"] - o.total_mass(u)) <= 1e-13 * o.total_mass(u)
        assert r4["load"] == r3["load"]
        assert r4["drift_rel_max"] <= DRIFT[F.FP64] and r4["steps"] == 4

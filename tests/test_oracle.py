"""The FP64 oracle against the reference's own element kernels and known answers (CPU)."""
import os

import numpy as np
import pytest

from eq_gb300 import workloads as wl
from oracle import hsld

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


# --- pins against the reference's generated kernels (fenics/hslD.h, boundary.h) ---
@pytest.fixture(scope="module")
def elements():
    return np.load(os.path.join(GOLDEN, "hsld_elements.npz"))


def test_bilinear_cell_tensor_matches_reference_kernel(elements):
    d = elements
    for t in range(len(d["D"])):
        A = hsld.element_a(d["coords"][t], d["D11"][t], d["D22"][t], d["D12"][t], d["D"][t],
                           d["dt"][t])
        assert _rel(A, d["a_cell"][t]) < 1e-13


def test_linear_cell_tensor_matches_reference_kernel(elements):
    d = elements
    for t in range(len(d["D"])):
        b = hsld.element_L(d["coords"][t], d["u0"][t], d["dt"][t], d["f"][t])
        assert _rel(b, d["L_cell"][t]) < 1e-13


def test_robin_facet_tensors_match_reference_kernels(elements):
    d = elements
    for t in range(len(d["D"])):
        A = hsld.facet_a(d["coords"][t], int(d["facet"][t]), d["dt"][t], d["r"][t])
        b = hsld.facet_L(d["coords"][t], int(d["facet"][t]), d["dt"][t], d["r"][t], d["s"][t])
        assert np.abs(A - d["a_facet"][t]).max() <= 1e-14 * max(1.0, np.abs(d["a_facet"][t]).max())
        assert np.abs(b - d["L_facet"][t]).max() <= 1e-14 * max(1.0, np.abs(d["L_facet"][t]).max())


def test_flux_facet_matches_reference_kernel(elements):
    d = elements
    for t in range(len(d["D"])):
        f = hsld.facet_flux(d["coords"][t], d["u0"][t], int(d["facet"][t]))
        assert abs(f - d["flux"][t]) <= 1e-12 * max(1.0, abs(d["flux"][t]))


def test_mesh_assembly_uses_the_pinned_element_tensors():
    """The assembled matrix equals the sum of element_a over the mesh triangles."""
    rng = np.random.default_rng(5)
    m = hsld.RightMesh(3.0, 2.0, 5, 3)
    D11, D22, D12 = rng.uniform(0.5, 1.5, (3, m.n_nodes))
    Ae = hsld.tabulate_a(m, 7.0, 0.2, D11, D22, D12)
    for t, cell in enumerate(m.cells):
        ref = hsld.element_a(m.coords[cell], D11[cell], D22[cell], D12[cell], 7.0, 0.2)
        assert _rel(Ae[t], ref) < 1e-13


def test_boundary_flux_integral_is_sum_of_facet_kernels():
    rng = np.random.default_rng(9)
    m = hsld.RightMesh(2.0, 1.5, 6, 4)
    u = rng.uniform(0, 1, m.n_nodes)
    total = 0.0
    for cell in m.cells:
        for facet in range(3):
            a, b = [cell[v] for v in range(3) if v != facet]
            xa, xb = m.coords[a], m.coords[b]
            on_bottom = xa[1] == 0 and xb[1] == 0
            on_top = np.isclose(xa[1], m.H) and np.isclose(xb[1], m.H)
            on_left = xa[0] == 0 and xb[0] == 0
            on_right = np.isclose(xa[0], m.W) and np.isclose(xb[0], m.W)
            if on_bottom or on_top or on_left or on_right:
                total += hsld.facet_flux(m.coords[cell], u[cell], facet)
    assert abs(hsld.boundary_flux_integral(m, u) - total) < 1e-12 * max(1.0, abs(total))


# --- analytic known answers ---
def test_interior_stencil_closed_form():
    o = hsld.HsldOracle(4.0, 2.0, 8, 4, D=3.0, dt=0.5, g=0.0, walls=0, factor=False)
    hx, hy, b = o.mesh.hx, o.mesh.hy, 1.5
    row = o.A.tocsr()[2 + 2 * 9].toarray().ravel()
    k = 2 + 2 * 9
    assert np.isclose(row[k], hx * hy / 2 + b * 2 * (hy / hx + hx / hy))
    assert np.isclose(row[k + 1], hx * hy / 12 - b * hy / hx)
    assert np.isclose(row[k + 9], hx * hy / 12 - b * hx / hy)
    assert np.isclose(row[k + 10], hx * hy / 12) and np.isclose(row[k - 10], hx * hy / 12)
    assert row[k + 8] == 0.0 and row[k - 8] == 0.0  # the other diagonal does not couple


def test_mass_is_conserved_with_zero_flux_walls():
    o = hsld.HsldOracle(5.0, 3.0, 20, 12, D=2.0, dt=0.1, g=0.0, walls=0)
    rng = np.random.default_rng(1)
    u = rng.uniform(0, 1, o.mesh.n_nodes)
    m0 = o.total_mass(u)
    for _ in range(10):
        u = o.step(u)
    assert abs(o.total_mass(u) - m0) < 1e-12 * m0


def test_uniform_field_decays_by_one_over_one_plus_dt_g():
    o = hsld.HsldOracle(5.0, 3.0, 10, 6, D=2.0, dt=0.1, g=0.5, walls=0)
    u = o.step(np.ones(o.mesh.n_nodes))
    assert np.allclose(u, 1.0 / (1.0 + 0.1 * 0.5), rtol=1e-12, atol=0)


def test_slowest_mode_decay_converges_to_continuum():
    """Dirichlet at y=0, zero flux elsewhere: slowest mode cos(0)*sin(pi y / 2H)."""
    W, H, D, dt = 4.0, 2.0, 1.0, 0.01
    lam = (np.pi / (2 * H)) ** 2
    errs = []
    for n in (8, 16, 32):
        o = hsld.HsldOracle(W, H, 2 * n, n, D=D, dt=dt, g=0.0, walls=1)
        y = o.mesh.coords[:, 1]
        u = np.sin(np.pi * y / (2 * H))
        for _ in range(50):
            u = o.step(u)
        u = o.step(u) / np.max(u)  # renormalised: now dominated by the slowest mode
        rate = np.max(u)
        errs.append(abs(rate - 1.0 / (1.0 + dt * D * lam)))
    assert errs[2] < errs[1] < errs[0]
    assert errs[1] / errs[2] > 3.0  # second order in h


def test_point_source_response_is_symmetric_under_half_turn():
    """A centred source on a right mesh with all walls Dirichlet: 180-degree symmetry."""
    o = hsld.HsldOracle(4.0, 4.0, 16, 16, D=1.0, dt=0.1, g=0.0, walls=15)
    F = hsld.point_load(o.mesh, np.array([[2.0, 2.0]]), np.array([1.0]), scale=0.1)
    u = o.step(np.zeros(o.mesh.n_nodes), F)
    U = u.reshape(17, 17)
    assert np.allclose(U, U[::-1, ::-1], rtol=0, atol=1e-14 * U.max())


def test_point_weights_partition_of_unity_and_exact_on_linear_fields():
    m = hsld.RightMesh(3.0, 2.0, 7, 5)
    rng = np.random.default_rng(3)
    xy = np.stack([rng.uniform(0, 3, 200), rng.uniform(0, 2, 200)], 1)
    nodes, w = hsld.point_weights(m, xy)
    assert np.allclose(w.sum(1), 1.0) and (w >= -1e-15).all()
    lin = 0.3 + 1.7 * m.coords[:, 0] - 0.9 * m.coords[:, 1]
    assert np.allclose(hsld.gather(m, lin, xy), 0.3 + 1.7 * xy[:, 0] - 0.9 * xy[:, 1])
    F = hsld.point_load(m, xy, np.ones(200), scale=0.5)
    assert np.isclose(F.sum(), 100.0)


def test_dirichlet_rows_hold_zero():
    o = hsld.HsldOracle(3.0, 2.0, 6, 4, D=1.0, dt=0.1, g=0.0, walls=1 | 8)
    F = hsld.point_load(o.mesh, np.array([[1.5, 1.0]]), np.array([2.0]), scale=0.1)
    u = o.step(np.zeros(o.mesh.n_nodes), F)
    assert np.all(u[o.dir] == 0.0) and u.max() > 0


# --- committed oracle fixtures (regression of the restatement itself) ---
def test_single_small_fixture_reproduces():
    d = np.load(os.path.join(GOLDEN, "single_small_oracle.npz"))
    trap = wl.single_small(0)
    assert np.array_equal(trap.cell_xy, d["xy"]) and np.array_equal(trap.cell_s, d["s"])
    out = hsld.run_trap(trap, steps=10, snapshots=(1, 10))
    for n in (1, 10):
        assert _rel(out["snapshots"][n][0], d[f"u_{n}"]) < 1e-12


def test_odd_mesh_fixture_reproduces():
    d = np.load(os.path.join(GOLDEN, "odd_mesh_oracle.npz"))
    for walls in (1, 0, 13):
        trap = wl.Trap(W=16.5, H=3.5, nx=33, ny=7, D=[49.0], g=[0.01], dt=0.1, steps=8,
                       walls=walls, cell_xy=d["xy"], cell_s=d["s"])
        out = hsld.run_trap(trap, steps=8)
        assert _rel(out["u"][0], d[f"u_walls{walls}"]) < 1e-12


def test_oracle_step_closes_its_mass_balance():
    """The balance identity on the oracle's own direct solve: the drift (free rows'
    residual sum) is rounding, the wall outflow is the consistent flux and agrees with
    the reference's facet functional up to the discretisation."""
    t = wl.single_small(0)
    o = hsld.HsldOracle(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)
    Fl = hsld.point_load(o.mesh, t.cell_xy, t.cell_s, scale=t.dt)
    u = np.zeros(o.mesh.n_nodes)
    for _ in range(30):
        un = o.step(u, Fl)
        bal = o.balance(un, u, Fl)
        u = un
        assert abs(bal["drift"]) <= 1e-12 * bal["mass"]
        lhs = bal["mass"] - bal["mass_prev"]
        rhs = bal["load"] - bal["decay"] - bal["operator_loss"] - bal["wall_outflow"]
        assert abs(lhs - rhs - bal["drift"]) <= 1e-12 * bal["mass"]
    assert bal["operator_loss"] == pytest.approx(0.0, abs=1e-12 * bal["mass"])
    assert abs(bal["load"] - t.dt * t.cell_s.sum()) <= 1e-12 * bal["load"]
    flux = o.boundary_flux(u)
    assert flux > 0 and abs(bal["wall_outflow"] - flux) <= 0.2 * flux


@pytest.mark.parametrize("name", ["single_large_oracle.npz", "two_species_oracle.npz",
                                  "batched_sample_oracle.npz"])
def test_config_fixtures_are_self_consistent(name):
    """The full-size fixtures: their cell values are the barycentric gather of their
    nodal fields at the workload's cells, and the batched sample is the stratified one."""
    g = np.load(os.path.join(GOLDEN, name))
    if name == "single_large_oracle.npz":
        t, pairs = wl.single_large(1), [("c0_500", "u0_500"), ("c0_50", "u0_50")]
    elif name == "two_species_oracle.npz":
        t, pairs = wl.two_species(2), [("c0_300", "u0_300"), ("c1_300", "u1_300")]
    else:
        traps = wl.batched_uneven(int(g["seed"]), int(g["n_traps"]))
        idx = [int(i) for i in g["traps"]]
        assert idx == wl.stratified_sample(traps, len(idx))
        t, pairs = traps[idx[-1]], [(f"t{idx[-1]}_c0_200", f"t{idx[-1]}_u0_200")]
    mesh = hsld.RightMesh(t.W, t.H, t.nx, t.ny)
    for c, u in pairs:
        assert g[u].shape == (t.n_nodes,)
        assert np.allclose(hsld.gather(mesh, g[u], t.cell_xy), g[c], rtol=1e-13, atol=0)
        assert np.all(np.isfinite(g[u])) and np.abs(g[u]).max() > 0


def test_left_diagonal_mesh_is_the_mirror_of_the_right_one():
    """The oracle's diagonal switch: the "left" triangulation is the "right" one mirrored
    in x, so a trap solved on it equals the mirrored trap on the "right" mesh (cells
    at W - x, left and right walls swapped, the tensor's D12 negated)."""
    W, H, nx, ny = 6.0, 3.0, 24, 12
    rng = np.random.Generator(np.random.PCG64(4))
    xy = np.stack([rng.uniform(0.2, W - 0.2, 15), rng.uniform(0.2, H - 0.2, 15)], 1)
    s = rng.uniform(0.5, 2.0, 15)
    n = (nx + 1) * (ny + 1)
    y, x = np.meshgrid(np.linspace(0, H, ny + 1), np.linspace(0, W, nx + 1), indexing="ij")
    th = 0.5 * np.sin(x) + 0.3 * y
    D11, D22, D12 = wl.rotated_tensor(th, 2.0, 0.5)
    mir = lambda a: np.asarray(a).reshape(ny + 1, nx + 1)[:, ::-1].ravel()  # noqa: E731
    walls = hsld.WALL_BOTTOM | hsld.WALL_LEFT
    left = hsld.HsldOracle(W, H, nx, ny, 49.0, 0.1, 0.01, walls, D11=D11.ravel(), D22=D22.ravel(),
                           D12=D12.ravel(), diagonal="left")
    right = hsld.HsldOracle(W, H, nx, ny, 49.0, 0.1, 0.01, hsld.WALL_BOTTOM | hsld.WALL_RIGHT,
                            D11=mir(D11), D22=mir(D22), D12=-mir(D12))
    xm = np.stack([W - xy[:, 0], xy[:, 1]], 1)
    Fl = hsld.point_load(left.mesh, xy, s, scale=0.1)
    Fr = hsld.point_load(right.mesh, xm, s, scale=0.1)
    ul, ur = np.zeros(n), np.zeros(n)
    for _ in range(4):
        ul, ur = left.step(ul, Fl), right.step(ur, Fr)
    assert np.allclose(ul, mir(ur), rtol=1e-12, atol=1e-14 * np.abs(ur).max())
    assert np.allclose(hsld.gather(left.mesh, ul, xy), hsld.gather(right.mesh, ur, xm), rtol=1e-12)
    assert abs(left.boundary_flux(ul) - right.boundary_flux(ur)) <= 1e-12 * abs(right.boundary_flux(ur))
    # and it is a different discretisation: the same trap on the two meshes differs
    same = hsld.HsldOracle(W, H, nx, ny, 49.0, 0.1, 0.01, walls, D11=D11.ravel(),
                           D22=D22.ravel(), D12=D12.ravel())
    ur2 = np.zeros(n)
    for _ in range(4):
        ur2 = same.step(ur2, hsld.point_load(same.mesh, xy, s, scale=0.1))
    assert np.linalg.norm(ur2 - ul) > 1e-6 * np.linalg.norm(ul)


def test_cpu_multigrid_baseline_solves_the_oracle_system():
    """The C/OpenMP multigrid-PCG CPU baseline (oracle/csrc/gmg_cpu.c) reaches the
    SuperLU solution of the same steps to the FP64 tolerance, on uneven traps with
    ragged coarse cells and on every wall set."""
    from oracle import gmg_cpu
    traps = [wl.single_small(0), wl.scaled(wl.single_small(0), 37, 19, n_cells=40)]
    for walls in (0, 13, 15):
        traps.append(wl.Trap(W=9.25, H=4.75, nx=37, ny=19, D=[490.0], g=[0.01], dt=0.1, steps=6,
                             walls=walls, cell_xy=traps[1].cell_xy, cell_s=traps[1].cell_s))
    out, dofs, _, _, its, tsec = gmg_cpu.run(traps, 6)
    assert dofs == 6 * sum(t.n_nodes for t in traps) and its > 0 and np.all(tsec > 0)
    for t, u in zip(traps, out):
        ref = hsld.run_trap(t, steps=6)["u"][0]
        assert np.linalg.norm(u - ref) <= 1e-9 * np.linalg.norm(ref)

"""The FP32 form with its refinement right-hand side and residual in FP64
(eqf_solver_opts.residual64 = 1, the plain form's kernels) instead of float pairs:
against the FP64 oracle at the chosen form's tolerance, on the 40x20 um trap, wall
values and a batch of uneven traps, and close to the pair-arithmetic default."""
import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import channel as chn
from oracle import hsld

pytestmark = pytest.mark.gpu
TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def tparams(t):
    return F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)


@pytest.mark.parametrize("use_graph", [0, 1])
def test_fp64_residual_variant_against_oracle(lib, use_graph):
    t = wl.single_small(0)
    ref = hsld.run_trap(t, steps=20)
    out = {}
    for r64 in (1, 0):
        with F.TrapBatch([tparams(t)], F.default_opts(F.FP32_IR, residual64=r64,
                                                      use_graph=use_graph)) as b:
            b.set_cells(0, t.cell_xy, t.cell_s)
            b.step(20)
            out[r64] = (b.read_nodal(0), b.read_cells(0), b.stats(0))
    u, c, st = out[1]
    assert rel(u, ref["u"][0]) <= TOL and rel(c, ref["cells"][0]) <= TOL
    assert st["last_rel_residual"] <= F.default_opts(F.FP32_IR).rtol
    assert rel(u, out[0][0]) <= TOL


def test_fp64_residual_variant_with_wall_values(lib):
    W, H, nx, ny = 10.0, 5.0, 40, 20
    walls = {chn.BOTTOM: (chn.DIRICHLET, 1.0, 0), chn.TOP: (chn.DIRICHLET, 2.0, 0),
             chn.LEFT: (chn.ROBIN, 0.5, 3.0)}
    tr = chn.MicrofluidicTrap(W, H, nx, ny, 490.0, 0.1, 0.01, walls, None)
    u = np.zeros(tr.mesh.n_nodes)
    for _ in range(6):
        u = tr.step(u, None)
    K = {chn.DIRICHLET: _lib.EQF_BC_DIRICHLET, chn.ROBIN: _lib.EQF_BC_ROBIN}
    tp = F.trap_params(W, H, nx, ny, 490.0, 0.1, 0.01, 0)
    with F.TrapBatch([tp], F.default_opts(F.FP32_IR, residual64=1)) as b:
        b.set_boundaries(0, {side: (K[k], v, r) for side, (k, v, r) in walls.items()})
        b.step(6)
        assert rel(b.read_nodal(0), u) <= TOL


def test_fp64_residual_variant_on_uneven_batch(lib):
    traps = wl.batched_uneven(3, 512)
    idx = [int(np.argmin([t.n_nodes for t in traps])), 17, 301]
    sub = [traps[i] for i in idx]
    refs = [hsld.run_trap(t, steps=10) for t in sub]
    with F.TrapBatch([tparams(t) for t in sub], F.default_opts(F.FP32_IR, residual64=1,
                                                              use_graph=1)) as b:
        for k, t in enumerate(sub):
            b.set_cells(k, t.cell_xy, t.cell_s)
        b.step(10)
        for k in range(len(sub)):
            assert rel(b.read_nodal(k), refs[k]["u"][0]) <= TOL
            assert rel(b.read_cells(k), refs[k]["cells"][0]) <= TOL

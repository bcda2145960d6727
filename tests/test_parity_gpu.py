"""GPU parity against the FP64 oracle, through the C ABI (include/eqfield.h)."""
import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import workloads as wl
from oracle import hsld

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_gpu(trap, steps, precision, **opts):
    tp = F.trap_params(trap.W, trap.H, trap.nx, trap.ny, trap.D[0], trap.dt, trap.g[0],
                       trap.walls)
    with F.TrapBatch([tp], F.default_opts(precision, **opts)) as b:
        b.set_cells(0, trap.cell_xy, trap.cell_s)
        b.step(steps)
        return b.read_nodal(0), b.read_cells(0), b.stats(0)


@pytest.mark.parametrize("precision,tol", [(F.FP64, 1e-9), (F.FP32_IR, 1e-6)])
def test_single_small_parity(lib, precision, tol):
    trap = wl.single_small(0)
    steps = 20
    ref = hsld.run_trap(trap, steps=steps)
    u, c, st = run_gpu(trap, steps, precision)
    assert rel(u, ref["u"][0]) <= tol, (rel(u, ref["u"][0]), st)
    assert rel(c, ref["cells"][0]) <= tol


@pytest.mark.parametrize("nx,ny", [(3, 2), (4, 4), (17, 9), (33, 7), (64, 32)])
@pytest.mark.parametrize("walls", [1, 0, 15, 1 | 4 | 8])
def test_small_meshes(lib, nx, ny, walls):
    trap = wl.Trap(W=nx * 0.5, H=ny * 0.5, nx=nx, ny=ny, D=[49.0], g=[0.01], dt=0.1, steps=5,
                   walls=walls)
    rng = np.random.default_rng(nx * 100 + ny)
    n = 7
    trap.cell_xy = np.stack([rng.uniform(0, trap.W, n), rng.uniform(0, trap.H, n)], 1)
    trap.cell_s = rng.lognormal(0, 0.5, n)
    ref = hsld.run_trap(trap, steps=5)
    u, c, st = run_gpu(trap, 5, F.FP64)
    assert rel(u, ref["u"][0]) <= 1e-9, st
    u32, c32, st32 = run_gpu(trap, 5, F.FP32_IR)
    assert rel(u32, ref["u"][0]) <= 1e-6, st32

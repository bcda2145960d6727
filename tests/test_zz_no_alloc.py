"""The allocation-free field integral against the ordinary readouts.

eqf_field_integral_noalloc serves callers that may not allocate device memory
when they need a mass-balance or boundary-flux figure (a simulation running under
its own device-memory budget, or code that must not trigger the synchronisation a
cudaMalloc/cudaFree can cause).  It keeps its reduction scratch in a fixed device
array inside the library instead of allocating per call.  This test checks it
through the C ABI against eqf_total_mass / eqf_boundary_flux on the same field,
on consecutive calls (which reuse the shared array), and that a field larger
than the stated maximum is refused.  The test allocates the field itself (with
torch); only the entry point under test must not allocate.
"""
import ctypes as C

import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # FP64 reductions of the same field in a different summation order


def _noalloc(lib, dev_ptr, trap, what, scale):
    out = C.c_double()
    rc = lib.eqf_field_integral_noalloc(C.c_void_p(dev_ptr), trap.nx, trap.ny, trap.W, trap.H,
                                        what, scale, None, C.byref(out))
    assert rc == _lib.EQF_OK, rc
    return out.value


def test_noalloc_integrals_match_batch_readouts(lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    trap = wl.single_small(0)
    tp = F.trap_params(trap.W, trap.H, trap.nx, trap.ny, trap.D[0], trap.dt, trap.g[0],
                       trap.walls)
    with F.TrapBatch([tp], F.default_opts(F.FP64)) as b:
        b.set_cells(0, trap.cell_xy, trap.cell_s)
        for steps in (5, 7):
            b.step(steps)
            u = b.read_nodal(0)
            mass_ref = b.total_mass(0)
            flux_ref = b.boundary_flux(0)
            dev = torch.from_numpy(u).to("cuda")
            torch.cuda.synchronize()
            # two calls in a row share the library's scratch array
            mass = _noalloc(lib, dev.data_ptr(), trap, 0, 1.0)
            flux = _noalloc(lib, dev.data_ptr(), trap, 1, trap.D[0] * trap.dt)
            assert abs(mass - mass_ref) <= RTOL * abs(mass_ref), (mass, mass_ref)
            assert abs(flux - flux_ref) <= RTOL * max(abs(flux_ref), 1e-300), (flux, flux_ref)
            assert mass_ref > 0.0 and flux_ref > 0.0


def test_noalloc_rejects_fields_beyond_its_maximum(lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = C.c_double(-1.0)
    side = int(np.sqrt(_lib.EQF_NOALLOC_MAX_NODES)) + 1  # (side+1)^2 nodes > maximum
    rc = lib.eqf_field_integral_noalloc(C.c_void_p(dev.data_ptr()), side, side, 1.0, 1.0, 0,
                                        1.0, None, C.byref(out))
    assert rc == _lib.EQF_ERR_TOO_LARGE
    assert out.value == -1.0

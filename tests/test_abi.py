"""The C ABI library without a GPU: it builds, loads, exports every declared symbol,
its structs match the header, and argument errors come back as status codes."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from eq_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "eqfield.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eqf_\w+)\s*\(", text)))


def test_header_declares_what_the_binding_knows():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_function(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (eqf_\w+)$", out, flags=re.M))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_struct_layout_matches_header():
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "eqfield.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(eqf_trap_params), offsetof(eqf_trap_params, walls),
         offsetof(eqf_trap_params, adv_len), offsetof(eqf_trap_params, dt));
  printf("%zu %zu %zu %zu\n", sizeof(eqf_solver_opts), offsetof(eqf_solver_opts, adaptive),
         offsetof(eqf_solver_opts, cheb_ratio), offsetof(eqf_solver_opts, inner_tol));
  printf("%zu %zu %zu %zu\n", sizeof(eqf_tune_bucket), offsetof(eqf_tune_bucket, tile_cols),
         offsetof(eqf_tune_bucket, dof_steps_per_s), offsetof(eqf_tune_bucket, max_sweeps));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), c, "-o", exe],
                       check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    tp = [int(v) for v in lines[0].split()]
    so = [int(v) for v in lines[1].split()]
    tb = [int(v) for v in lines[2].split()]
    T, S = _lib.TrapParams, _lib.SolverOpts
    assert tp == [C.sizeof(T), T.walls.offset, T.adv_len.offset, T.dt.offset]
    assert so == [C.sizeof(S), S.adaptive.offset, S.cheb_ratio.offset, S.inner_tol.offset]
    B = _lib.TuneBucket
    assert tb == [C.sizeof(B), B.tile_cols.offset, B.dof_steps_per_s.offset, B.max_sweeps.offset]


def test_default_opts_without_gpu(lib):
    o = _lib.SolverOpts()
    assert lib.eqf_default_opts(_lib.EQF_PREC_FP32_IR, C.byref(o)) == _lib.EQF_OK
    assert o.precision == _lib.EQF_PREC_FP32_IR and o.rtol > 0 and o.max_iters >= 1
    assert lib.eqf_default_opts(7, C.byref(o)) == _lib.EQF_ERR_INVALID


def test_invalid_arguments_are_status_codes(lib):
    h = C.c_void_p()
    o = _lib.SolverOpts()
    lib.eqf_default_opts(_lib.EQF_PREC_FP64, C.byref(o))
    assert lib.eqf_create(0, None, C.byref(o), C.byref(h)) == _lib.EQF_ERR_INVALID
    assert b"trap" in lib.eqf_last_error(None)
    bad = (_lib.TrapParams * 1)(_lib.TrapParams(1.0, 1.0, 0, 4, 1.0, 0.1, 0.0, 0.0, 1.0, 1))
    assert lib.eqf_create(1, bad, C.byref(o), C.byref(h)) == _lib.EQF_ERR_INVALID
    assert lib.eqf_step(None, 1) == _lib.EQF_ERR_INVALID
    assert lib.eqf_destroy(None) == _lib.EQF_ERR_INVALID


def test_create_reports_missing_device(lib):
    """On a machine without a GPU the library refuses loudly (no CPU fallback)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    h = C.c_void_p()
    o = _lib.SolverOpts()
    lib.eqf_default_opts(_lib.EQF_PREC_FP64, C.byref(o))
    tp = (_lib.TrapParams * 1)(_lib.TrapParams(4.0, 2.0, 8, 4, 1.0, 0.1, 0.0, 0.0, 1.0, 1))
    rc = lib.eqf_create(1, tp, C.byref(o), C.byref(h))
    assert rc in (_lib.EQF_ERR_NO_DEVICE, _lib.EQF_ERR_CUDA)
    assert lib.eqf_last_error(None)


def test_noalloc_rejects_oversize_before_touching_a_device(lib):
    out = C.c_double(-1.0)
    rc = lib.eqf_field_integral_noalloc(C.c_void_p(16), 4096, 4096, 1.0, 1.0, 0, 1.0, None,
                                        C.byref(out))
    assert rc == _lib.EQF_ERR_TOO_LARGE and out.value == -1.0
    assert lib.eqf_field_integral_noalloc(None, 4, 4, 1.0, 1.0, 0, 1.0, None,
                                          C.byref(out)) == _lib.EQF_ERR_INVALID


SERVE_HEADER = os.path.join(ROOT, "include", "eqserve.h")


def test_serving_header_matches_binding_and_exports(lib):
    from eq_gb300 import serve
    text = re.sub(r"/\*.*?\*/", "", open(SERVE_HEADER).read(), flags=re.S)
    declared = sorted(set(re.findall(r"\b(eqs_\w+)\s*\(", text)))
    assert declared == sorted(serve.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (eqs_\w+)$", out, flags=re.M))
    assert not [f for f in declared if f not in exported]


def test_serving_struct_layout_matches_header():
    from eq_gb300 import serve
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "eqserve.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(eqs_config), offsetof(eqs_config, hbm_budget),
         offsetof(eqs_config, max_wait_ms), offsetof(eqs_config, steps_in_flight),
         offsetof(eqs_config, reuse_slots));
  printf("%zu %zu %zu %zu\n", sizeof(eqs_request), offsetof(eqs_request, n_cells),
         offsetof(eqs_request, vmax), offsetof(eqs_request, want_nodal));
  printf("%zu %zu\n", sizeof(eqs_result_info), offsetof(eqs_result_info, cohort));
  printf("%zu %zu %zu\n", sizeof(eqs_stats), offsetof(eqs_stats, bytes_peak),
         offsetof(eqs_stats, slot_admitted));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), c, "-o", exe],
                       check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = [[int(v) for v in ln.split()] for ln in lines[:4]]
    S = serve
    assert got[0] == [C.sizeof(S.ServerConfig), S.ServerConfig.hbm_budget.offset,
                      S.ServerConfig.max_wait_ms.offset, S.ServerConfig.steps_in_flight.offset,
                      S.ServerConfig.reuse_slots.offset]
    assert got[1] == [C.sizeof(S.Request), S.Request.n_cells.offset, S.Request.vmax.offset,
                      S.Request.want_nodal.offset]
    assert got[2] == [C.sizeof(S.ResultInfo), S.ResultInfo.cohort.offset]
    assert got[3] == [C.sizeof(S.Stats), S.Stats.bytes_peak.offset, S.Stats.slot_admitted.offset]


def test_serving_without_a_device_reports_no_device(lib):
    from eq_gb300 import serve
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    cfg = serve.default_config()
    h = C.c_void_p()
    assert serve._bind(lib).eqs_create(C.byref(cfg), C.byref(h)) == _lib.EQF_ERR_NO_DEVICE


def test_footprint_estimate_needs_no_device(lib):
    from eq_gb300 import field as F
    t = F.trap_params(40.0, 20.0, 160, 80, 490.0, 0.1, 0.01)
    small = F.footprint_estimate([t], F.default_opts(F.FP32_IR), 300)
    big = F.footprint_estimate([t, t], F.default_opts(F.FP64), 600)
    assert 13041 * 60 < small < 13041 * 400
    assert big > 2 * small

"""ctypes binding of the C ABI in include/eqfield.h (``eq_gb300/libeqfield.so``).

The CUDA library is the only implementation: if it is missing this module raises,
and there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeqfield.so")

EQF_OK = 0
EQF_ERR_INVALID = -1
EQF_ERR_CUDA = -2
EQF_ERR_NOT_CONVERGED = -3
EQF_ERR_NO_DEVICE = -4
EQF_ERR_NOMEM = -5
EQF_ERR_TOO_LARGE = -6
EQF_NOALLOC_MAX_NODES = 8388608

EQF_WALL_BOTTOM, EQF_WALL_TOP, EQF_WALL_LEFT, EQF_WALL_RIGHT = 1, 2, 4, 8
EQF_PREC_FP64, EQF_PREC_FP32_IR = 0, 1
EQF_KRYLOV_AUTO, EQF_KRYLOV_CG, EQF_KRYLOV_BICGSTAB = 0, 1, 2

# every entry point declared in include/eqfield.h
EXPORTS = (
    "eqf_default_opts", "eqf_create", "eqf_destroy", "eqf_last_error", "eqf_num_nodes",
    "eqf_set_cells", "eqf_set_cell_rates", "eqf_set_nodal", "eqf_add_nodal", "eqf_step",
    "eqf_read_nodal", "eqf_read_cells", "eqf_boundary_flux", "eqf_total_mass", "eqf_stats",
    "eqf_sync", "eqf_set_cell_rates_all", "eqf_read_cells_all", "eqf_profile",
    "eqf_profile_read", "eqf_stream", "eqf_field_integral_noalloc", "eqf_couple_species",
    "eqf_poll", "eqf_read_cells_async", "eqf_read_nodal_async", "eqf_set_active",
    "eqf_replace_trap", "eqf_replace_traps", "eqf_slot_fits",
    "eqf_footprint_estimate", "eqf_fail_count_async", "eqf_create_tuned", "eqf_autotune",
    "eqf_set_rods", "eqf_update_rods", "eqf_read_rods", "eqf_exchange_rods", "eqf_rod_waves",
    "eqf_update_rods_all", "eqf_read_rods_all",
    "eqf_set_boundaries", "eqf_read_channels", "eqf_set_channels", "eqf_set_well",
    "eqf_read_well", "eqf_set_tensor", "eqf_trap_info", "eqf_json_open", "eqf_json_frame", "eqf_json_frame_host",
    "eqf_json_close", "eqf_vtk_open", "eqf_vtk_write", "eqf_vtk_write_channel",
    "eqf_vtk_write_host", "eqf_vtk_close", "eqf_mass_balance", "eqf_read_balance",
    "eqf_read_nodal_dof", "eqf_set_nodal_dof", "eqf_set_well_concentration",
    "eqf_autotune_log",
    "eqf_rod_relax_passes",
)

# wall conditions (eqf_set_boundaries)
EQF_SIDE_BOTTOM, EQF_SIDE_TOP, EQF_SIDE_LEFT, EQF_SIDE_RIGHT = 0, 1, 2, 3
EQF_BC_NEUMANN, EQF_BC_DIRICHLET, EQF_BC_ROBIN, EQF_BC_CHANNEL, EQF_BC_WELL = 0, 1, 2, 3, 4
PROF_CLASSES = ("smooth0", "smooth0_first", "resid0", "restrict0", "prolong0", "coarse",
                "cg_dir", "cg_update", "ir_resid_first", "ir_resid", "ir_update", "scalar",
                "down0", "up0", "rod_exchange", "balance", "down0_cg")

# rod cells (eqf_set_rods): per cell and layer modes, and the eqf_rod record
EQF_MAX_ROD_LAYERS = 4
EQF_ROD_HELD, EQF_ROD_CIRCUIT, EQF_ROD_INERT = 0, 1, 2


class Balance(C.Structure):
    """eqf_balance: the last step's FP64 mass-balance terms and the sums since enabled."""
    _fields_ = [(n, C.c_double) for n in (
        "mass", "mass_prev", "load", "decay", "operator_loss", "wall_outflow", "drift",
        "drift_sum", "drift_abs_sum", "load_sum", "drift_rel_max")] + [("steps", C.c_int64)]


class TrapParams(C.Structure):
    _fields_ = [("width", C.c_double), ("height", C.c_double), ("nx", C.c_int32),
                ("ny", C.c_int32), ("D", C.c_double), ("dt", C.c_double), ("decay", C.c_double),
                ("adv_u", C.c_double), ("adv_len", C.c_double), ("walls", C.c_uint32)]


class SolverOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("rtol", C.c_double), ("max_sweeps", C.c_int32),
                ("max_iters", C.c_int32), ("inner_tol", C.c_double), ("cheb_pre", C.c_int32),
                ("cheb_post", C.c_int32), ("cheb_coarse", C.c_int32), ("cheb_ratio", C.c_double),
                ("use_graph", C.c_int32), ("adaptive", C.c_int32),
                ("tile_nodes", C.c_int32), ("krylov", C.c_int32), ("fuse_levels", C.c_int32),
                ("residual64", C.c_int32), ("tile_cols", C.c_int32)]


class TuneBucket(C.Structure):
    _fields_ = [("max_nodes", C.c_int64), ("tile_nodes", C.c_int32), ("cheb_pre", C.c_int32),
                ("cheb_post", C.c_int32), ("tile_cols", C.c_int32),
                ("dof_steps_per_s", C.c_double), ("max_iters", C.c_int32),
                ("max_sweeps", C.c_int32)]


EQF_TUNE_MAX_BUCKETS = 8


class TuneTable(C.Structure):
    _fields_ = [("n", C.c_int32), ("b", TuneBucket * EQF_TUNE_MAX_BUCKETS)]


class Wall(C.Structure):
    _fields_ = [("kind", C.c_int32), ("value", C.c_double), ("rate", C.c_double)]


class Boundaries(C.Structure):
    _fields_ = [("wall", Wall * 4), ("channel_velocity", C.c_double), ("channel_D", C.c_double),
                ("channel_rate", C.c_double * 2), ("channel_substeps", C.c_int32),
                ("well_scaling", C.c_double)]


class RodLaw(C.Structure):
    _fields_ = [("nodes_per_micron", C.c_double), ("dt", C.c_double),
                ("membrane_rate", C.c_double * EQF_MAX_ROD_LAYERS)]


def rod_dtype():
    """numpy record layout of eqf_rod (20 doubles, 160 bytes)."""
    import numpy as np
    return np.dtype([("center", "<f8", (2,)), ("pole_a", "<f8", (2,)), ("pole_b", "<f8", (2,)),
                     ("body_pos", "<f8", (2,)), ("body_rot", "<f8", (2,)), ("verts", "<f8", (8,)),
                     ("length", "<f8"), ("reserved", "<f8")])


class EqfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"eqfield error {code}: {msg}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m eq_gb300.build` "
                           "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    dp, i64p = P(C.c_double), P(C.c_int64)
    sig = {
        "eqf_default_opts": (C.c_int, [C.c_int32, P(SolverOpts)]),
        "eqf_create": (C.c_int, [C.c_int32, P(TrapParams), P(SolverOpts), P(C.c_void_p)]),
        "eqf_destroy": (C.c_int, [C.c_void_p]),
        "eqf_last_error": (C.c_char_p, [C.c_void_p]),
        "eqf_num_nodes": (C.c_int, [C.c_void_p, C.c_int32, i64p]),
        "eqf_set_cells": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp, dp]),
        "eqf_set_cell_rates": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp]),
        "eqf_set_nodal": (C.c_int, [C.c_void_p, C.c_int32, dp]),
        "eqf_add_nodal": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, i64p, dp]),
        "eqf_step": (C.c_int, [C.c_void_p, C.c_int32]),
        "eqf_read_nodal": (C.c_int, [C.c_void_p, C.c_int32, dp]),
        "eqf_read_cells": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp]),
        "eqf_boundary_flux": (C.c_int, [C.c_void_p, C.c_int32, dp]),
        "eqf_total_mass": (C.c_int, [C.c_void_p, C.c_int32, dp]),
        "eqf_stats": (C.c_int, [C.c_void_p, C.c_int32, i64p, i64p, i64p, dp]),
        "eqf_sync": (C.c_int, [C.c_void_p]),
        "eqf_set_cell_rates_all": (C.c_int, [C.c_void_p, C.c_int64, dp]),
        "eqf_read_cells_all": (C.c_int, [C.c_void_p, C.c_int64, dp]),
        "eqf_profile": (C.c_int, [C.c_void_p, C.c_int32]),
        "eqf_stream": (C.c_int, [C.c_void_p, P(C.c_void_p)]),
        "eqf_field_integral_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double,
                                                 C.c_double, C.c_int32, C.c_double, C.c_void_p,
                                                 dp]),
        "eqf_profile_read": (C.c_int, [C.c_void_p, C.c_int32, dp, i64p, i64p, dp]),
        "eqf_couple_species": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, P(C.c_int32),
                                         C.c_double, C.c_double, C.c_double]),
        "eqf_poll": (C.c_int, [C.c_void_p, P(C.c_int32)]),
        "eqf_read_cells_async": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp]),
        "eqf_read_nodal_async": (C.c_int, [C.c_void_p, C.c_int32, dp]),
        "eqf_set_active": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
        "eqf_replace_trap": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(TrapParams)]),
        "eqf_replace_traps": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                        C.POINTER(TrapParams)]),
        "eqf_slot_fits": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(TrapParams),
                                    C.POINTER(C.c_int32)]),
        "eqf_fail_count_async": (C.c_int, [C.c_void_p, P(C.c_int32)]),
        "eqf_create_tuned": (C.c_int, [C.c_int32, P(TrapParams), P(SolverOpts), P(TuneTable),
                                       P(C.c_void_p)]),
        "eqf_autotune": (C.c_int, [C.c_int32, P(TrapParams), P(SolverOpts), C.c_double,
                                   P(TuneTable)]),
        "eqf_autotune_log": (C.c_int, [C.c_int32, P(TrapParams), P(SolverOpts), C.c_double,
                                       P(TuneTable), C.c_char_p, C.c_int64]),
        "eqf_footprint_estimate": (C.c_int, [C.c_int32, P(TrapParams), P(SolverOpts), C.c_int64,
                                             i64p]),
        "eqf_set_rods": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_int32), P(RodLaw), C.c_int64,
                                   C.c_void_p, dp, dp, P(C.c_uint8)]),
        "eqf_update_rods": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, dp]),
        "eqf_read_rods": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp, dp, P(C.c_int32)]),
        "eqf_update_rods_all": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, dp]),
        "eqf_read_rods_all": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, P(C.c_int32)]),
        "eqf_exchange_rods": (C.c_int, [C.c_void_p]),
        "eqf_set_boundaries": (C.c_int, [C.c_void_p, C.c_int32, P(Boundaries)]),
        "eqf_read_channels": (C.c_int, [C.c_void_p, C.c_int32, dp, dp]),
        "eqf_set_channels": (C.c_int, [C.c_void_p, C.c_int32, dp, dp]),
        "eqf_set_well": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double]),
        "eqf_trap_info": (C.c_int, [C.c_void_p, C.c_int32, P(TrapParams)]),
        "eqf_set_tensor": (C.c_int, [C.c_void_p, C.c_int32, dp, dp, dp]),
        "eqf_json_open": (C.c_int, [C.c_char_p, C.c_int64, C.c_int32, C.c_int32,
                                    P(C.c_void_p)]),
        "eqf_json_frame": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, P(C.c_int32), C.c_double,
                                     C.c_int64, dp, C.c_int64, i64p, C.c_int32, dp]),
        "eqf_json_frame_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp, C.c_double,
                                          C.c_int64, dp, C.c_int64, i64p, C.c_int32, dp]),
        "eqf_json_close": (C.c_int, [C.c_void_p, C.c_char_p]),
        "eqf_vtk_open": (C.c_int, [C.c_char_p, P(C.c_void_p)]),
        "eqf_vtk_write": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_double]),
        "eqf_vtk_write_channel": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                            C.c_double]),
        "eqf_vtk_write_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int32,
                                         C.c_int32, dp, C.c_double]),
        "eqf_vtk_close": (C.c_int, [C.c_void_p]),
        "eqf_read_well": (C.c_int, [C.c_void_p, C.c_int32, dp, i64p]),
        "eqf_rod_waves": (C.c_int, [C.c_void_p, P(C.c_int32)]),
        "eqf_rod_relax_passes": (C.c_int, [C.c_void_p, P(C.c_int32)]),
        "eqf_mass_balance": (C.c_int, [C.c_void_p, C.c_int32]),
        "eqf_read_balance": (C.c_int, [C.c_void_p, C.c_int32, P(Balance)]),
        "eqf_read_nodal_dof": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_int32), dp]),
        "eqf_set_nodal_dof": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_int32), dp]),
        "eqf_set_well_concentration": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib

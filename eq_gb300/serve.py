"""ctypes mirror of the serving loop in include/eqserve.h (continuous batching of
trap-simulation requests over eqfield cohorts).  The loop itself is native code
(eq_gb300/csrc/eqf_server.cu); this module only marshals requests and results."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import EqfError, SolverOpts, TrapParams

EXPORTS = ("eqs_default_config", "eqs_create", "eqs_destroy", "eqs_last_error", "eqs_submit",
           "eqs_progress", "eqs_take_done", "eqs_result", "eqs_get_stats", "eqs_drain")


class ServerConfig(C.Structure):
    _fields_ = [("opts", SolverOpts), ("hbm_budget", C.c_int64), ("max_cohorts", C.c_int32),
                ("max_cohort_traps", C.c_int32), ("min_batch", C.c_int32),
                ("max_wait_ms", C.c_double), ("steps_in_flight", C.c_int32),
                ("reuse_slots", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("species", TrapParams * 2), ("n_species", C.c_int32), ("n_cells", C.c_int64),
                ("xy", C.POINTER(C.c_double)), ("s", C.POINTER(C.c_double)),
                ("sender", C.POINTER(C.c_int32)), ("vmax", C.c_double), ("K", C.c_double),
                ("uptake", C.c_double), ("steps", C.c_int32), ("want_nodal", C.c_int32)]


class ResultInfo(C.Structure):
    _fields_ = [("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("steps", C.c_int32), ("status", C.c_int32), ("n_nodes", C.c_int64),
                ("n_cells", C.c_int64), ("n_species", C.c_int32), ("cohort", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("failed", C.c_int64), ("cohorts", C.c_int64), ("pending", C.c_int64),
                ("running", C.c_int64), ("dof_steps", C.c_double), ("busy_s", C.c_double),
                ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double),
                ("step_ms_p999", C.c_double), ("step_samples", C.c_int64),
                ("bytes_in_use", C.c_int64), ("bytes_peak", C.c_int64),
                ("admit_s", C.c_double), ("launch_s", C.c_double), ("release_s", C.c_double),
                ("first_step_s", C.c_double), ("readout_s", C.c_double),
                ("slot_admitted", C.c_int64), ("fill_s", C.c_double),
                ("fills", C.c_int64), ("refill_step_s", C.c_double)]


def _bind(lib):
    if getattr(lib, "_eqs_bound", False):
        return lib
    P = C.POINTER
    sig = {
        "eqs_default_config": (C.c_int, [P(ServerConfig)]),
        "eqs_create": (C.c_int, [P(ServerConfig), P(C.c_void_p)]),
        "eqs_destroy": (C.c_int, [C.c_void_p]),
        "eqs_last_error": (C.c_char_p, [C.c_void_p]),
        "eqs_submit": (C.c_int, [C.c_void_p, P(Request), P(C.c_int64)]),
        "eqs_progress": (C.c_int, [C.c_void_p]),
        "eqs_take_done": (C.c_int, [C.c_void_p, P(C.c_int64), C.c_int32, P(C.c_int32)]),
        "eqs_result": (C.c_int, [C.c_void_p, C.c_int64, P(C.c_double), P(C.c_double),
                                 P(ResultInfo)]),
        "eqs_get_stats": (C.c_int, [C.c_void_p, P(Stats)]),
        "eqs_drain": (C.c_int, [C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._eqs_bound = True
    return lib


def default_config(**over) -> ServerConfig:
    lib = _bind(_lib.load())
    c = ServerConfig()
    rc = lib.eqs_default_config(C.byref(c))
    if rc:
        raise EqfError(rc, "eqs_default_config")
    for k, v in over.items():
        if hasattr(c.opts, k):
            setattr(c.opts, k, v)
        elif hasattr(c, k):
            setattr(c, k, v)
        else:
            raise KeyError(k)
    return c


@dataclass
class Result:
    id: int
    cells: np.ndarray            # (n_species, n_cells)
    nodal: Optional[np.ndarray]  # (n_species, n_nodes) when asked for
    t_submit: float
    t_admit: float
    t_done: float
    steps: int
    status: int
    cohort: int


class Server:
    """One serving loop (single host thread)."""

    def __init__(self, config: Optional[ServerConfig] = None):
        self._lib = _bind(_lib.load())
        self._h = C.c_void_p()
        cfg = config if config is not None else default_config()
        rc = self._lib.eqs_create(C.byref(cfg), C.byref(self._h))
        if rc:
            raise EqfError(rc, "eqs_create")
        self._meta: Dict[int, tuple] = {}

    def _ck(self, rc):
        if rc:
            msg = self._lib.eqs_last_error(self._h)
            raise EqfError(rc, msg.decode() if msg else "")

    def close(self):
        if self._h:
            self._lib.eqs_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, species: Sequence[TrapParams], xy: np.ndarray, s: np.ndarray, steps: int,
               sender: Optional[np.ndarray] = None, vmax: float = 0.5, K: float = 0.1,
               uptake: float = 0.05, want_nodal: bool = False) -> int:
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        s = np.ascontiguousarray(s, dtype=np.float64).ravel()
        r = Request()
        ns = len(species)
        if ns not in (1, 2):
            raise ValueError("one or two species")
        for k in range(ns):
            r.species[k] = species[k]
        r.n_species = ns
        r.n_cells = len(s)
        r.xy = xy.ctypes.data_as(C.POINTER(C.c_double))
        r.s = s.ctypes.data_as(C.POINTER(C.c_double))
        snd = None
        if ns == 2:
            snd = np.ascontiguousarray(sender, dtype=np.int32).ravel()
            r.sender = snd.ctypes.data_as(C.POINTER(C.c_int32))
        r.vmax, r.K, r.uptake = float(vmax), float(K), float(uptake)
        r.steps = int(steps)
        r.want_nodal = 1 if want_nodal else 0
        rid = C.c_int64()
        self._ck(self._lib.eqs_submit(self._h, C.byref(r), C.byref(rid)))
        nodes = (species[0].nx + 1) * (species[0].ny + 1)
        self._meta[rid.value] = (ns, len(s), nodes, want_nodal)
        return rid.value

    def last_error(self) -> str:
        msg = self._lib.eqs_last_error(self._h)
        return msg.decode() if msg else ""

    def progress(self):
        self._ck(self._lib.eqs_progress(self._h))

    def drain(self):
        self._ck(self._lib.eqs_drain(self._h))

    def take_done(self, cap: int = 4096) -> List[int]:
        ids = (C.c_int64 * cap)()
        n = C.c_int32()
        self._ck(self._lib.eqs_take_done(self._h, ids, cap, C.byref(n)))
        return [ids[i] for i in range(n.value)]

    def result(self, rid: int) -> Result:
        ns, nc, nodes, want = self._meta.pop(rid)
        cells = np.zeros((ns, nc))
        nodal = np.zeros((ns, nodes)) if want else None
        info = ResultInfo()
        self._ck(self._lib.eqs_result(
            self._h, rid, cells.ctypes.data_as(C.POINTER(C.c_double)),
            nodal.ctypes.data_as(C.POINTER(C.c_double)) if want else None, C.byref(info)))
        return Result(rid, cells, nodal, info.t_submit, info.t_admit, info.t_done, info.steps,
                      info.status, info.cohort)

    def stats(self) -> Dict[str, float]:
        st = Stats()
        self._ck(self._lib.eqs_get_stats(self._h, C.byref(st)))
        return {name: getattr(st, name) for name, _ in Stats._fields_}

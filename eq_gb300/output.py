"""Writers of the reference's output formats (ctypes mirror of eqf_json_* / eqf_vtk_*).

JsonRecording mirrors jsonRecording (src/main.cpp:81-192: init / recordFrame /
finalize); VtkSeries mirrors the DOLFIN File series of
fenicsInterface::writeDiffusionFiles (src/fHSL.cpp:606-632).  Both write from the C
library; the batch-reading forms read the fields from the GPU.
"""
from __future__ import annotations

import ctypes as C
import json
from typing import Optional, Sequence

import numpy as np

from . import _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ck(rc, what):
    if rc != _lib.EQF_OK:
        raise _lib.EqfError(rc, what)


class JsonRecording:
    """One simulation's JSON recording (format v00_02)."""

    def __init__(self, path: str, time_since_epoch: int = 0, node_id: int = 0,
                 sim_number: int = 0):
        self._lib = _lib.load()
        self._h = C.c_void_p()
        _ck(self._lib.eqf_json_open(path.encode(), int(time_since_epoch), int(node_id),
                                    int(sim_number), C.byref(self._h)), "cannot open " + path)

    @staticmethod
    def _cells(ids, data):
        ids = np.ascontiguousarray(ids if ids is not None else np.zeros((0, 2)),
                                   dtype=np.int64).reshape(-1, 2)
        n = len(ids)
        data = np.ascontiguousarray(data if data is not None else np.zeros((n, 0)),
                                    dtype=np.float64)
        data = data.reshape(n, data.size // n if n else 0)
        return ids, data

    def frame(self, sim_time: float, batch=None, layers: Sequence[int] = (),
              fields: Optional[np.ndarray] = None, divisions=None, ids=None, data=None):
        """One frame: externalHSL from the batch's layers, or from `fields`
        (n_layers x n_nodes, grid order); divisions (n x 5), cell ids (n x 2: id,
        strain type) and data (n x k: x, y, angle, length, spring, HSL nM ...)."""
        ids, data = self._cells(ids, data)
        div = np.ascontiguousarray(divisions if divisions is not None else np.zeros((0, 5)),
                                   dtype=np.float64).reshape(-1, 5)
        i64 = C.POINTER(C.c_int64)
        if batch is not None:
            lay = np.ascontiguousarray(layers, dtype=np.int32)
            rc = self._lib.eqf_json_frame(self._h, batch._h, len(lay),
                                          lay.ctypes.data_as(C.POINTER(C.c_int32)),
                                          float(sim_time), len(div), _dp(div), len(ids),
                                          ids.ctypes.data_as(i64), data.shape[1], _dp(data))
        else:
            f = np.ascontiguousarray(fields if fields is not None else np.zeros((0, 0)),
                                     dtype=np.float64)
            f = f.reshape(f.shape[0], -1) if f.ndim == 2 else f.reshape(1, -1)
            rc = self._lib.eqf_json_frame_host(self._h, f.shape[0], f.shape[1], _dp(f),
                                               float(sim_time), len(div), _dp(div), len(ids),
                                               ids.ctypes.data_as(i64), data.shape[1], _dp(data))
        _ck(rc, "json frame")

    def close(self, parameters: Optional[dict] = None):
        if self._h:
            text = json.dumps(parameters, sort_keys=True) if parameters is not None else None
            _ck(self._lib.eqf_json_close(self._h, text.encode() if text else None), "json close")
            self._h = None


class VtkSeries:
    """A .pvd series of field snapshots."""

    def __init__(self, pvd_path: str):
        self._lib = _lib.load()
        self._h = C.c_void_p()
        _ck(self._lib.eqf_vtk_open(pvd_path.encode(), C.byref(self._h)), "cannot open " + pvd_path)

    def write(self, batch, trap: int, time: float):
        _ck(self._lib.eqf_vtk_write(self._h, batch._h, int(trap), float(time)), "vtk write")

    def write_channel(self, batch, trap: int, side: int, time: float):
        _ck(self._lib.eqf_vtk_write_channel(self._h, batch._h, int(trap), int(side), float(time)),
            "vtk channel")

    def write_host(self, width: float, height: float, nx: int, ny: int, field, time: float):
        f = np.ascontiguousarray(field, dtype=np.float64)
        _ck(self._lib.eqf_vtk_write_host(self._h, float(width), float(height), int(nx), int(ny),
                                         _dp(f), float(time)), "vtk write")

    def close(self):
        if self._h:
            self._lib.eqf_vtk_close(self._h)
            self._h = None

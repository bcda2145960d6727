"""ctypes loader of the plain-C rod-coupling restatement (oracle/csrc/rods_port.c).

TEST/BENCH INFRASTRUCTURE ONLY (the timed CPU baseline of the rod exchange and a
second restatement pinned against the reference's code).  build() compiles it with
gcc into oracle/librods_port.so (git-ignored), on whichever host runs it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "rods_port.c")
LIB = os.path.join(HERE, "librods_port.so")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-shared", "-fPIC", "-o",
                        LIB + ".tmp", SRC, "-lm"], check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        dp = C.POINTER(C.c_double)
        lib.rods_port_exchange.restype = C.c_int
        lib.rods_port_exchange.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, dp, C.c_int,
                                           C.c_int, dp, dp, dp, C.POINTER(C.c_uint8), dp, dp,
                                           C.POINTER(C.c_int)]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Exchanger:
    """Holds the C-contiguous state of one colony for repeated passes."""

    def __init__(self, fields, rods, ihsl, prod, mode, npm, dt, km):
        self.f = np.ascontiguousarray(fields, dtype=np.float64).copy()
        self.nl, ny1, nx1 = self.f.shape
        self.nx, self.ny = nx1 - 1, ny1 - 1
        self.r = np.ascontiguousarray(rods).view(np.float64).reshape(-1, 20).copy()
        self.n = self.r.shape[0]
        self.ih = np.ascontiguousarray(ihsl, dtype=np.float64).reshape(self.n, self.nl).copy()
        self.pr = np.ascontiguousarray(prod, dtype=np.float64).reshape(self.n, self.nl).copy()
        self.md = np.ascontiguousarray(mode, dtype=np.uint8).reshape(self.n, self.nl).copy()
        self.km = np.ascontiguousarray(km, dtype=np.float64)[:self.nl].copy()
        self.npm, self.dt = float(npm), float(dt)
        self.eh = np.zeros((self.n, self.nl))
        self.pts = np.zeros(self.n, dtype=np.int32)

    def run(self):
        rc = load().rods_port_exchange(
            self.nx, self.ny, self.npm, self.dt, _p(self.km), self.nl, self.n, _p(self.r),
            _p(self.ih), _p(self.pr), self.md.ctypes.data_as(C.POINTER(C.c_uint8)), _p(self.f),
            _p(self.eh), self.pts.ctypes.data_as(C.POINTER(C.c_int)))
        if rc != 0:
            raise RuntimeError("footprint larger than the lattice")

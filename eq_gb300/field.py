"""Host-side mirror of eQ's diffusion-solver plugin over the CUDA C ABI.

``TrapBatch`` is a thin object wrapper of include/eqfield.h (one handle = many
independent traps).  ``FieldSolver`` mirrors the reference's plugin interface
``eQ::diffusionSolver`` (src/eQ.h:302-330) as implemented by ``fenicsInterface``
(src/fHSL.h:333-449): ``initDiffusion(params)``, ``stepDiffusion()``,
``getBoundaryFlux()``, ``writeDiffusionFiles(t)``, ``finalize()`` and the
``solution_vector`` / ``totalBoundaryFlux`` data plane that
``Simulation::stepSimulation`` reads and writes (src/simulation.cpp:455-505).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import EqfError, SolverOpts, TrapParams

WALL_BOTTOM, WALL_TOP, WALL_LEFT, WALL_RIGHT = 1, 2, 4, 8
FP64, FP32_IR = _lib.EQF_PREC_FP64, _lib.EQF_PREC_FP32_IR
KRYLOV_AUTO, KRYLOV_CG, KRYLOV_BICGSTAB = (_lib.EQF_KRYLOV_AUTO, _lib.EQF_KRYLOV_CG,
                                           _lib.EQF_KRYLOV_BICGSTAB)

# trapType -> Dirichlet walls under boundaryType DIRICHLET_0 (src/fHSL.cpp:557-569)
TRAP_TYPES = {"NOWALLED": 15, "THREEWALLED": WALL_BOTTOM, "TWOWALLED": WALL_BOTTOM | WALL_TOP,
              "ONEWALLED": WALL_BOTTOM | WALL_LEFT | WALL_RIGHT}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(lib, h, rc):
    if rc != _lib.EQF_OK:
        msg = lib.eqf_last_error(h)
        raise EqfError(rc, msg.decode() if msg else "")


def default_opts(precision: int = FP64, **over) -> SolverOpts:
    lib = _lib.load()
    o = SolverOpts()
    _check(lib, None, lib.eqf_default_opts(precision, C.byref(o)))
    for k, v in over.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def footprint_estimate(traps: Sequence[TrapParams], opts: Optional[SolverOpts] = None,
                       n_cells: int = 0) -> int:
    """Device bytes a batch of these traps would hold (eqf_footprint_estimate)."""
    lib = _lib.load()
    arr = (TrapParams * len(traps))(*traps)
    out = C.c_int64()
    rc = lib.eqf_footprint_estimate(len(traps), arr, C.byref(opts) if opts is not None else None,
                                    int(n_cells), C.byref(out))
    _check(lib, None, rc)
    return out.value


def trap_params(W, H, nx, ny, D, dt, decay=0.0, walls=WALL_BOTTOM, adv_u=0.0,
                adv_len=1.0) -> TrapParams:
    return TrapParams(float(W), float(H), int(nx), int(ny), float(D), float(dt), float(decay),
                      float(adv_u), float(adv_len), int(walls))


def autotune(traps: Sequence[TrapParams], opts: Optional[SolverOpts] = None,
             budget_s: float = 20.0) -> _lib.TuneTable:
    """Per size bucket, the fastest tile node target, 2-D tile width, Chebyshev
    degrees and Krylov schedule (eqf_autotune_log; runs on the GPU for about budget_s
    seconds at most).  The returned table carries every measured candidate in .log."""
    lib = _lib.load()
    arr = (TrapParams * len(traps))(*traps)
    table = _lib.TuneTable()
    buf = C.create_string_buffer(1 << 16)
    rc = lib.eqf_autotune_log(len(traps), arr, C.byref(opts) if opts is not None else None,
                              float(budget_s), C.byref(table), buf, len(buf))
    _check(lib, None, rc)
    table.log = [dict(zip(("bucket", "tile_nodes", "tile_cols", "cheb_pre", "cheb_post",
                           "max_iters", "max_sweeps", "dof_steps_per_s"),
                          (float(x) for x in ln.split())))
                 for ln in buf.value.decode().splitlines() if ln.strip()]
    return table


def tune_table_dict(table: _lib.TuneTable) -> List[Dict[str, float]]:
    return [{"max_nodes": table.b[i].max_nodes, "tile_nodes": table.b[i].tile_nodes,
             "tile_cols": table.b[i].tile_cols, "cheb_pre": table.b[i].cheb_pre,
             "cheb_post": table.b[i].cheb_post, "max_iters": table.b[i].max_iters,
             "max_sweeps": table.b[i].max_sweeps, "dof_steps_per_s": table.b[i].dof_steps_per_s}
            for i in range(table.n)]


class TrapBatch:
    """A batch of independent traps on the GPU (C ABI handle).  With a tuning table
    (autotune) the traps take their size bucket's tile target and the batch its
    dominant bucket's smoother degrees and Krylov schedule."""

    def __init__(self, traps: Sequence[TrapParams], opts: Optional[SolverOpts] = None,
                 tune: Optional[_lib.TuneTable] = None):
        self._lib = _lib.load()
        arr = (TrapParams * len(traps))(*traps)
        self._h = C.c_void_p()
        o = opts if opts is not None else default_opts()
        if tune is not None:
            rc = self._lib.eqf_create_tuned(len(traps), arr, C.byref(o), C.byref(tune),
                                            C.byref(self._h))
        else:
            rc = self._lib.eqf_create(len(traps), arr, C.byref(o), C.byref(self._h))
        _check(self._lib, None, rc)
        self.n_traps = len(traps)
        self.params = list(traps)
        self.opts = o
        self._ncells = [0] * self.n_traps

    def close(self):
        if getattr(self, "_h", None):
            self._lib.eqf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        _check(self._lib, self._h, rc)

    def num_nodes(self, trap: int) -> int:
        n = C.c_int64()
        self._ck(self._lib.eqf_num_nodes(self._h, trap, C.byref(n)))
        return n.value

    def set_cells(self, trap: int, xy: np.ndarray, s: np.ndarray):
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        s = np.ascontiguousarray(s, dtype=np.float64).ravel()
        if len(s) != len(xy):
            raise ValueError("xy and s lengths differ")
        self._ck(self._lib.eqf_set_cells(self._h, trap, len(s), _dp(xy), _dp(s)))
        self._ncells[trap] = len(s)

    def couple_species(self, trap1: int, trap2: int, sender: np.ndarray, vmax: float = 0.5,
                       K: float = 0.1, uptake: float = 0.05):
        """Sender/receiver pair: species 1 on trap1 (cells and senders' rates from
        set_cells(trap1, ...)), species 2 on trap2 (same mesh; gets the same cells)."""
        snd = np.ascontiguousarray(sender, dtype=np.int32).ravel()
        if len(snd) != self._ncells[trap1]:
            raise ValueError("one sender flag per cell of trap1")
        self._ck(self._lib.eqf_couple_species(self._h, trap1, trap2,
                                              snd.ctypes.data_as(C.POINTER(C.c_int32)),
                                              float(vmax), float(K), float(uptake)))
        self._ncells[trap2] = len(snd)

    def set_cell_rates(self, trap: int, s: np.ndarray):
        s = np.ascontiguousarray(s, dtype=np.float64).ravel()
        self._ck(self._lib.eqf_set_cell_rates(self._h, trap, len(s), _dp(s)))

    def set_nodal(self, trap: int, c: np.ndarray):
        c = np.ascontiguousarray(c, dtype=np.float64).ravel()
        if len(c) != self.num_nodes(trap):
            raise ValueError("nodal vector length mismatch")
        self._ck(self._lib.eqf_set_nodal(self._h, trap, _dp(c)))

    def add_nodal(self, trap: int, nodes: np.ndarray, delta: np.ndarray):
        nodes = np.ascontiguousarray(nodes, dtype=np.int64).ravel()
        delta = np.ascontiguousarray(delta, dtype=np.float64).ravel()
        if len(nodes) != len(delta):
            raise ValueError("nodes and delta lengths differ")
        self._ck(self._lib.eqf_add_nodal(self._h, trap, len(nodes),
                                         nodes.ctypes.data_as(C.POINTER(C.c_int64)), _dp(delta)))

    def step(self, n: int = 1):
        self._ck(self._lib.eqf_step(self._h, int(n)))

    # --- wall conditions and flow channels (eqf_set_boundaries) ----------------------
    def set_boundaries(self, trap: int, walls: Dict[int, tuple],
                       channel: Optional[dict] = None):
        """walls[side] = (kind, value, rate) by _lib.EQF_SIDE_* (missing sides: Neumann);
        channel = {"velocity", "D", "rate": (left, right), "substeps", "well_scaling"}."""
        bc = _lib.Boundaries()
        for side in range(4):
            kind, value, rate = walls.get(side, (_lib.EQF_BC_NEUMANN, 0.0, 0.0))
            bc.wall[side].kind = int(kind)
            bc.wall[side].value = float(value)
            bc.wall[side].rate = float(rate)
        ch = channel or {}
        bc.channel_velocity = float(ch.get("velocity", 0.0))
        bc.channel_D = float(ch.get("D", 0.0))
        rates = ch.get("rate", (0.0, 0.0))
        bc.channel_rate[0] = float(rates[0])
        bc.channel_rate[1] = float(rates[1])
        bc.channel_substeps = int(ch.get("substeps", 1))
        bc.well_scaling = float(ch.get("well_scaling", 1.0))
        self._ck(self._lib.eqf_set_boundaries(self._h, int(trap), C.byref(bc)))

    def read_channels(self, trap: int, bottom: bool = True, top: bool = True):
        nx = self.params[trap].nx
        b = np.empty(nx + 1) if bottom else None
        t = np.empty(nx + 1) if top else None
        self._ck(self._lib.eqf_read_channels(self._h, int(trap), _dp(b) if b is not None else None,
                                             _dp(t) if t is not None else None))
        return b, t

    def set_channels(self, trap: int, bottom: Optional[np.ndarray] = None,
                     top: Optional[np.ndarray] = None):
        b = None if bottom is None else np.ascontiguousarray(bottom, dtype=np.float64)
        t = None if top is None else np.ascontiguousarray(top, dtype=np.float64)
        self._ck(self._lib.eqf_set_channels(self._h, int(trap), _dp(b) if b is not None else None,
                                            _dp(t) if t is not None else None))

    def set_tensor(self, trap: int, D11=None, D22=None, D12=None):
        """Per-node anisotropic tensor (grid order); None restores the isotropic one."""
        if D11 is None:
            self._ck(self._lib.eqf_set_tensor(self._h, int(trap), None, None, None))
            return
        a, b_, c = (np.ascontiguousarray(v, dtype=np.float64).ravel() for v in (D11, D22, D12))
        n = self.num_nodes(trap)
        if not (len(a) == len(b_) == len(c) == n):
            raise ValueError("one tensor value per node")
        self._ck(self._lib.eqf_set_tensor(self._h, int(trap), _dp(a), _dp(b_), _dp(c)))

    def set_well(self, trap: int, well_scaling: float, decay_rate: float):
        """Boundary well of a trap (0 scaling: off); walls of kind EQF_BC_WELL take it."""
        self._ck(self._lib.eqf_set_well(self._h, int(trap), float(well_scaling),
                                        float(decay_rate)))

    def read_well(self, trap: int):
        c = C.c_double()
        u = C.c_int64()
        self._ck(self._lib.eqf_read_well(self._h, int(trap), C.byref(c), C.byref(u)))
        return c.value, u.value

    # --- rod cells of the agent-based model (eqf_set_rods) -----------------------
    def set_rods(self, layers: Sequence[int], rods: np.ndarray, ihsl: np.ndarray,
                 production: np.ndarray, mode: np.ndarray, nodes_per_micron: float,
                 dt: float, membrane_rate: Sequence[float]):
        """Rod cells (records of ``_lib.rod_dtype()``) coupled to the layers ``layers``
        the reference's way; ihsl / production / mode are (n_cells, n_layers)."""
        nl = len(layers)
        lay = np.ascontiguousarray(layers, dtype=np.int32)
        rods = np.ascontiguousarray(rods, dtype=_lib.rod_dtype())
        n = len(rods)
        ih = np.ascontiguousarray(ihsl, dtype=np.float64).reshape(n, nl)
        pr = np.ascontiguousarray(production, dtype=np.float64).reshape(n, nl)
        md = np.ascontiguousarray(mode, dtype=np.uint8).reshape(n, nl)
        law = _lib.RodLaw()
        law.nodes_per_micron = float(nodes_per_micron)
        law.dt = float(dt)
        for l, k in enumerate(membrane_rate):
            law.membrane_rate[l] = float(k)
        self._ck(self._lib.eqf_set_rods(
            self._h, nl, lay.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(law), n,
            rods.ctypes.data if n else None, _dp(ih), _dp(pr),
            md.ctypes.data_as(C.POINTER(C.c_uint8))))
        self._rods = getattr(self, "_rods", {})
        self._rods[int(layers[0])] = (n, nl)

    def update_rods(self, layer0: int, rods: np.ndarray,
                    production: Optional[np.ndarray] = None):
        rods = np.ascontiguousarray(rods, dtype=_lib.rod_dtype())
        pr = None
        if production is not None:
            pr = _dp(np.ascontiguousarray(production, dtype=np.float64).ravel())
        self._ck(self._lib.eqf_update_rods(self._h, int(layer0), len(rods), rods.ctypes.data,
                                           pr))

    def read_rods(self, layer0: int):
        """(ihsl, ehsl, points): intracellular HSL (molecules) and the last gathered
        footprint mean per cell and layer, and the footprint size per cell."""
        n, nl = self._rods[int(layer0)]
        ih = np.empty((n, nl))
        eh = np.empty((n, nl))
        pts = np.empty(n, dtype=np.int32)
        self._ck(self._lib.eqf_read_rods(self._h, int(layer0), n, _dp(ih), _dp(eh),
                                         pts.ctypes.data_as(C.POINTER(C.c_int32))))
        return ih, eh, pts

    def _rod_sets(self):
        """(first layer, cells, layers) of every rod set, in increasing first layer."""
        return [(l0, n, nl) for l0, (n, nl) in sorted(getattr(self, "_rods", {}).items())
                if n > 0]

    def update_rods_all(self, rods: np.ndarray, production: Optional[np.ndarray] = None):
        """update_rods for every rod set in one call: the sets' cells in turn, in
        increasing order of their first layer (production: each set's block laid out
        as for update_rods)."""
        rods = np.ascontiguousarray(rods, dtype=_lib.rod_dtype())
        pr = None
        if production is not None:
            pr = _dp(np.ascontiguousarray(production, dtype=np.float64).ravel())
        self._ck(self._lib.eqf_update_rods_all(self._h, len(rods), rods.ctypes.data, pr))

    def read_rods_all(self):
        """read_rods for every rod set in one call: lists of each set's (ihsl, ehsl,
        points), in increasing order of the sets' first layer."""
        sets = self._rod_sets()
        tot = sum(n for _, n, _ in sets)
        totp = sum(n * nl for _, n, nl in sets)
        ih = np.empty(totp)
        eh = np.empty(totp)
        pts = np.empty(tot, dtype=np.int32)
        self._ck(self._lib.eqf_read_rods_all(self._h, tot, _dp(ih), _dp(eh),
                                             pts.ctypes.data_as(C.POINTER(C.c_int32))))
        out, c0, p0 = [], 0, 0
        for _, n, nl in sets:
            out.append((ih[p0:p0 + n * nl].reshape(n, nl), eh[p0:p0 + n * nl].reshape(n, nl),
                        pts[c0:c0 + n]))
            c0 += n
            p0 += n * nl
        return out

    def exchange_rods(self):
        """One pass of the cell loop without a solve."""
        self._ck(self._lib.eqf_exchange_rods(self._h))

    def rod_waves(self) -> int:
        w = C.c_int32()
        self._ck(self._lib.eqf_rod_waves(self._h, C.byref(w)))
        return w.value

    def rod_relax_passes(self) -> int:
        p = C.c_int32()
        self._ck(self._lib.eqf_rod_relax_passes(self._h, C.byref(p)))
        return p.value

    def read_nodal(self, trap: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.num_nodes(trap))
        self._ck(self._lib.eqf_read_nodal(self._h, trap, _dp(out)))
        return out

    def read_nodal_dof(self, trap: int, dof_from_vertex: np.ndarray) -> np.ndarray:
        """The nodal field in a DOF order: out[dof_from_vertex[v]] = field(v)."""
        dof = np.ascontiguousarray(dof_from_vertex, dtype=np.int32)
        out = np.empty(self.num_nodes(trap))
        self._ck(self._lib.eqf_read_nodal_dof(self._h, trap,
                                              dof.ctypes.data_as(C.POINTER(C.c_int32)), _dp(out)))
        return out

    def set_nodal_dof(self, trap: int, dof_from_vertex: np.ndarray, c: np.ndarray):
        dof = np.ascontiguousarray(dof_from_vertex, dtype=np.int32)
        c = np.ascontiguousarray(c, dtype=np.float64)
        self._ck(self._lib.eqf_set_nodal_dof(self._h, trap,
                                             dof.ctypes.data_as(C.POINTER(C.c_int32)), _dp(c)))

    def set_well_concentration(self, trap: int, c: float):
        self._ck(self._lib.eqf_set_well_concentration(self._h, trap, float(c)))

    def read_cells(self, trap: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        n = self._ncells[trap]
        if out is None:
            out = np.empty(n)
        self._ck(self._lib.eqf_read_cells(self._h, trap, n, _dp(out)))
        return out

    def boundary_flux(self, trap: int) -> float:
        v = C.c_double()
        self._ck(self._lib.eqf_boundary_flux(self._h, trap, C.byref(v)))
        return v.value

    def total_mass(self, trap: int) -> float:
        v = C.c_double()
        self._ck(self._lib.eqf_total_mass(self._h, trap, C.byref(v)))
        return v.value

    def set_active(self, trap: int, active: bool):
        """Freezes (False) or resumes (True) a trap (eqf_set_active)."""
        self._ck(self._lib.eqf_set_active(self._h, int(trap), 1 if active else 0))

    def replace_trap(self, trap: int, params: TrapParams):
        """Reuses trap slot `trap` for a new trap whose grid fits it (eqf_replace_trap);
        the new trap starts empty: set its cells afterwards."""
        self.replace_traps([trap], [params])

    def slot_fits(self, trap: int, params: TrapParams) -> bool:
        """Whether replace_trap(trap, params) would accept the grid (eqf_slot_fits)."""
        ok = C.c_int32()
        self._ck(self._lib.eqf_slot_fits(self._h, int(trap), C.byref(params), C.byref(ok)))
        return bool(ok.value)

    def replace_traps(self, traps: Sequence[int], params: Sequence[TrapParams]):
        """Several slots at once (eqf_replace_traps: one rebuild)."""
        tr = (C.c_int32 * len(traps))(*[int(t) for t in traps])
        pp = (TrapParams * len(params))(*params)
        self._ck(self._lib.eqf_replace_traps(self._h, len(traps), tr, pp))
        for t, p in zip(traps, params):
            self._ncells[t] = 0
            self.params[t] = p

    def mass_balance(self, enable: bool = True):
        """Per-step FP64 mass balance of every trap (eqf_mass_balance); enabling zeroes
        the sums."""
        self._ck(self._lib.eqf_mass_balance(self._h, 1 if enable else 0))

    def read_balance(self, trap: int) -> Dict[str, float]:
        """The last step's balance terms of a trap and the sums since enabled."""
        out = _lib.Balance()
        self._ck(self._lib.eqf_read_balance(self._h, trap, C.byref(out)))
        return {name: getattr(out, name) for name, _ in _lib.Balance._fields_}

    def stats(self, trap: int) -> Dict[str, float]:
        st, sw, it = C.c_int64(), C.c_int64(), C.c_int64()
        rr = C.c_double()
        self._ck(self._lib.eqf_stats(self._h, trap, C.byref(st), C.byref(sw), C.byref(it),
                                     C.byref(rr)))
        return {"steps": st.value, "sweeps": sw.value, "iters": it.value,
                "last_rel_residual": rr.value}

    def sync(self):
        self._ck(self._lib.eqf_sync(self._h))

    @property
    def n_cells_total(self) -> int:
        return int(sum(self._ncells))

    def set_cell_rates_all(self, s: np.ndarray):
        s = np.ascontiguousarray(s, dtype=np.float64).ravel()
        self._ck(self._lib.eqf_set_cell_rates_all(self._h, len(s), _dp(s)))

    def read_cells_all(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.n_cells_total)
        self._ck(self._lib.eqf_read_cells_all(self._h, len(out), _dp(out)))
        return out

    def stream_handle(self) -> int:
        """cudaStream_t of the batch as an integer (for external CUDA events)."""
        v = C.c_void_p()
        self._ck(self._lib.eqf_stream(self._h, C.byref(v)))
        return int(v.value or 0)

    def profile(self, enable: bool):
        self._ck(self._lib.eqf_profile(self._h, 1 if enable else 0))

    def profile_read(self) -> Dict[str, Dict[str, float]]:
        n = len(_lib.PROF_CLASSES)
        ms = np.zeros(n)
        bts = np.zeros(n)
        la = np.zeros(n, dtype=np.int64)
        nd = np.zeros(n, dtype=np.int64)
        i64 = C.POINTER(C.c_int64)
        self._ck(self._lib.eqf_profile_read(self._h, n, _dp(ms), la.ctypes.data_as(i64),
                                            nd.ctypes.data_as(i64), _dp(bts)))
        return {name: {"ms": float(ms[i]), "launches": int(la[i]), "nodes": int(nd[i]),
                       "bytes": float(bts[i])} for i, name in enumerate(_lib.PROF_CLASSES)}


@dataclass
class DiffusionParams:
    """The fields of eQ::diffusionSolver::params (src/eQ.h:305-321) the field step uses."""
    dt: float
    D_HSL: float
    trapWidthMicrons: float
    trapHeightMicrons: float
    nodesPerMicron: float
    uniqueID: int = 0
    filePath: str = ""
    trapChannelVelocity: float = 0.0


class FieldSolver:
    """One HSL layer behind the reference's plugin interface.

    Mesh sizes follow fenicsClassInit: nodesW = ceil(W*npm), nodesH = ceil(H*npm)
    squares (src/fHSL.cpp:242-243).  The default walls are the THREEWALLED
    DIRICHLET_0 trap.  ``solution_vector`` is a grid-order numpy array; as in the
    reference the caller may modify it between steps (deposits), and
    ``stepDiffusion`` pushes it to the device, steps and pulls it back.
    """

    def __init__(self, trapType: str = "THREEWALLED", decay: float = 0.0,
                 precision: int = FP64, opts: Optional[SolverOpts] = None):
        self.walls = TRAP_TYPES[trapType]
        self.decay = decay
        self.precision = precision
        self.opts = opts
        self.batch: Optional[TrapBatch] = None
        self.solution_vector = np.zeros(0)
        self.totalBoundaryFlux = 0.0
        self.myParams: Optional[DiffusionParams] = None
        self._pushed = None

    def initDiffusion(self, params: DiffusionParams):
        self.myParams = params
        nx = int(math.ceil(params.trapWidthMicrons * params.nodesPerMicron))
        ny = int(math.ceil(params.trapHeightMicrons * params.nodesPerMicron))
        tp = trap_params(params.trapWidthMicrons, params.trapHeightMicrons, nx, ny,
                         params.D_HSL, params.dt, self.decay, self.walls)
        o = self.opts if self.opts is not None else default_opts(self.precision)
        self.batch = TrapBatch([tp], o)
        self.nodesW, self.nodesH = nx + 1, ny + 1
        self.solution_vector = np.zeros(self.nodesW * self.nodesH)
        self._pushed = self.solution_vector.copy()

    def stepDiffusion(self):
        if not np.array_equal(self.solution_vector, self._pushed):
            self.batch.set_nodal(0, self.solution_vector)
        self.batch.step(1)
        self.solution_vector = self.batch.read_nodal(0)
        self._pushed = self.solution_vector.copy()
        self.totalBoundaryFlux = self.batch.boundary_flux(0)

    def getBoundaryFlux(self) -> Dict[str, float]:
        return {"totalFlux": self.totalBoundaryFlux}

    def writeDiffusionFiles(self, timestamp: float):
        """Nodal snapshot in grid order (the reference writes DOLFIN .pvd files)."""
        if not self.myParams or not self.myParams.filePath:
            return
        base = os.path.splitext(self.myParams.filePath)[0]
        with open(f"{base}_{timestamp:.6g}.json", "w") as f:
            json.dump({"time": timestamp, "nodesW": self.nodesW, "nodesH": self.nodesH,
                       "externalHSL": self.solution_vector.tolist()}, f)

    def finalize(self):
        if self.batch is not None:
            self.batch.close()
            self.batch = None

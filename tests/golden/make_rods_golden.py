"""Generates tests/golden/rods_reference.npz: the reference's own rod-cell coupling
(eQabm::updateCells' footprint search, readHSL, membrane exchange and writeHSL,
compiled from the reference sources by oracle/ref_rods.py) on seeded cases.

Cases (each three passes of the cell loop, the state of one pass feeding the next):

* ``colony``    20x10 um at 2 nodes/um, 70 random rods (overlaps allowed), two
                layers, senders / receivers / strains without a circuit.
* ``walls``     20x10 um at 4 nodes/um: short rods (no interior node: centre-node
                fallback) and rods hugging the walls (clamped poles, clamped search).
* ``grown``     16x8 um at 2.5 nodes/um: separated body halves and ratchet-grown boxes,
                quarter-turn rotations given exactly.
* ``lattice``   12x6 um at 2 nodes/um: axis-aligned rods whose box edges lie on lattice
                lines (the strict inside test excludes them).
* ``stack``     10x6 um at 2 nodes/um, three layers: rods piled on one spot (a long
                chain of cells sharing nodes).

Run from the repository root (needs the reference sources):
    python tests/golden/make_rods_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from eq_gb300 import workloads as wl  # noqa: E402
from oracle import ref_rods  # noqa: E402

PASSES = 3


def _modes(rng, n, nl):
    mode = np.full((n, nl), wl.ROD_HELD, dtype=np.uint8)
    mode[:, 0] = wl.ROD_CIRCUIT
    inert = rng.uniform(size=n) < 0.15
    mode[inert, :] = wl.ROD_INERT
    return mode


def case_colony(rng):
    W, H, npm, nl, n = 20.0, 10.0, 2.0, 2, 70
    rods = wl.rod_records(rng.uniform(1.0, W - 1.0, n), rng.uniform(1.0, H - 1.0, n),
                          rng.uniform(0.0, 2 * np.pi, n), rng.uniform(1.2, 4.5, n), W, H)
    return W, H, npm, nl, rods


def case_walls(rng):
    W, H, npm, nl, n = 20.0, 10.0, 4.0, 2, 60
    short = n // 2
    cx = np.concatenate([rng.uniform(0.5, W - 0.5, short),
                         rng.choice([0.05, W - 0.05], n - short) + rng.uniform(-0.04, 0.04, n - short)])
    cy = np.concatenate([rng.uniform(0.5, H - 0.5, short), rng.uniform(0.0, H, n - short)])
    cx, cy = np.clip(cx, 0.0, W), np.clip(cy, 0.0, H)
    length = np.concatenate([rng.uniform(1.0, 1.15, short), rng.uniform(2.0, 4.0, n - short)])
    rods = wl.rod_records(cx, cy, rng.uniform(0.0, np.pi, n), length, W, H)
    return W, H, npm, nl, rods


def case_grown(rng):
    W, H, npm, nl, n = 16.0, 8.0, 2.5, 2, 40
    cx, cy = rng.uniform(2.0, W - 2.0, n), rng.uniform(2.0, H - 2.0, n)
    length = rng.uniform(2.0, 4.0, n)
    ang = rng.uniform(0.0, 2 * np.pi, n)
    rods = wl.rod_records(cx, cy, ang, length, W, H)
    quarter = np.arange(n) % 4 == 0
    rods["body_rot"][quarter] = np.array([0.0, 1.0])
    # separated halves: body A behind the centre along the axis; ratchet-grown box
    sep = rng.uniform(0.0, 0.6, n)
    rot = rods["body_rot"]
    rods["body_pos"][:, 0] = cx - rot[:, 0] * sep * 0.5
    rods["body_pos"][:, 1] = cy - rot[:, 1] * sep * 0.5
    grow = rng.uniform(0.0, 0.5, n)
    rods["verts"][:, 2] += grow
    rods["verts"][:, 4] += grow
    return W, H, npm, nl, rods


def case_lattice(rng):
    W, H, npm, nl = 12.0, 6.0, 2.0, 2
    cx = np.array([2.0, 4.5, 6.0, 8.0, 3.0, 9.5, 5.0, 7.25])
    cy = np.array([2.0, 2.5, 4.0, 3.5, 4.5, 1.5, 1.0, 5.0])
    length = np.array([2.0, 3.0, 2.5, 3.5, 1.5, 2.0, 4.0, 2.0])
    ang = np.zeros(len(cx))
    rods = wl.rod_records(cx, cy, ang, length, W, H)
    rods["body_rot"] = np.array([1.0, 0.0])
    vert = np.arange(len(cx)) % 2 == 1
    rods["body_rot"][vert] = np.array([0.0, 1.0])
    for k in np.nonzero(vert)[0]:  # poles along y for the vertical ones
        L = length[k]
        for key, r in (("pole_a", 1.0), ("pole_b", -1.0)):
            kk = r * 0.5 * L - 0.5
            rods[key][k] = [np.clip(cx[k], 0, W), np.clip(cy[k] + kk, 0, H)]
    return W, H, npm, nl, rods


def case_stack(rng):
    W, H, npm, nl, n = 10.0, 6.0, 2.0, 3, 24
    cx = 5.0 + rng.uniform(-0.6, 0.6, n)
    cy = 3.0 + rng.uniform(-0.6, 0.6, n)
    rods = wl.rod_records(cx, cy, rng.uniform(0.0, np.pi, n), rng.uniform(2.0, 4.0, n), W, H)
    return W, H, npm, nl, rods


CASES = {"colony": case_colony, "walls": case_walls, "grown": case_grown,
         "lattice": case_lattice, "stack": case_stack}


def main(path=os.path.join(HERE, "rods_reference.npz")):
    if ref_rods.build_if_available() is None:
        raise SystemExit("reference sources not found: cannot regenerate " + path)
    out = {}
    for ci, (name, make) in enumerate(CASES.items()):
        rng = np.random.Generator(np.random.PCG64(4100 + ci))
        W, H, npm, nl, rods = make(rng)
        n = len(rods)
        nx, ny = int(W * npm), int(H * npm)
        fields = rng.uniform(0.0, 50.0, (nl, ny + 1, nx + 1))
        ihsl = rng.uniform(0.0, 3000.0, (n, nl))
        prod = np.zeros((n, nl))
        prod[:, 0] = np.where(rng.uniform(size=n) < 0.5, 120.0, 0.0)
        mode = _modes(rng, n, nl)
        dt = 0.1
        km = [3.0, 2.1, 1.7][:nl]
        out[f"{name}/geom"] = np.array([W, H, npm, dt])
        out[f"{name}/km"] = np.array(km)
        out[f"{name}/rods"] = np.ascontiguousarray(rods).view(np.float64).reshape(n, 20)
        out[f"{name}/fields_in"] = fields
        out[f"{name}/ihsl_in"] = ihsl
        out[f"{name}/prod"] = prod
        out[f"{name}/mode"] = mode
        f, ih = fields, ihsl
        for p in range(PASSES):
            f, ih, eh, pts = ref_rods.exchange(f, rods, ih, prod, mode, npm, dt, km)
            out[f"{name}/ehsl_{p}"] = eh
            out[f"{name}/ihsl_{p}"] = ih
        out[f"{name}/fields_out"] = f
        out[f"{name}/points"] = pts
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()

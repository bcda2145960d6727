"""Generates the golden fixtures under tests/golden/.

* hsld_elements.npz — element tensors of the reference's own generated kernels
  (fenics/hslD.h, fenics/boundary.h), compiled here by oracle/ref_kernels.py from
  the reference sources, on seeded random triangles and coefficients: bilinear
  cell (anisotropic tensor), Robin facets, linear cell and facets, flux facet.
* single_small_oracle.npz — the FP64 oracle on the 160x80-square trap (300 cells,
  seed 0): nodal field and cell concentrations after steps 1, 10 and 100.
* odd_mesh_oracle.npz — the oracle on a 33x7 trap with three wall sets.

Run from the repository root (needs the reference sources for the first file):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from eq_gb300 import workloads as wl  # noqa: E402
from oracle import hsld, ref_kernels  # noqa: E402


def element_fixture(path):
    if ref_kernels.build_if_available() is None:
        raise SystemExit("reference sources not found: cannot regenerate " + path)
    rng = np.random.Generator(np.random.PCG64(2024))
    n = 64
    coords = np.empty((n, 3, 2))
    for t in range(n):
        if t % 4 == 0:  # a lower-right "right" triangle
            hx, hy = rng.uniform(0.05, 2.0, 2)
            x0, y0 = rng.uniform(-5, 5, 2)
            coords[t] = [[x0, y0], [x0 + hx, y0], [x0 + hx, y0 + hy]]
        elif t % 4 == 1:  # an upper-left "right" triangle
            hx, hy = rng.uniform(0.05, 2.0, 2)
            x0, y0 = rng.uniform(-5, 5, 2)
            coords[t] = [[x0, y0], [x0, y0 + hy], [x0 + hx, y0 + hy]]
        else:  # a general positively oriented triangle
            while True:
                c = rng.uniform(-3, 3, (3, 2))
                det = (c[1, 0] - c[0, 0]) * (c[2, 1] - c[0, 1]) - (c[2, 0] - c[0, 0]) * (c[1, 1] - c[0, 1])
                if abs(det) > 0.5:
                    coords[t] = c if det > 0 else c[[0, 2, 1]]
                    break
    D11 = rng.uniform(0.2, 2.0, (n, 3))
    D22 = rng.uniform(0.2, 2.0, (n, 3))
    D12 = rng.uniform(-0.3, 0.3, (n, 3))
    D = rng.uniform(1.0, 500.0, n)
    dt = rng.uniform(0.01, 0.2, n)
    u0 = rng.uniform(-1.0, 2.0, (n, 3))
    f = rng.uniform(-1.0, 1.0, n)
    r = rng.uniform(0.0, 3.0, n)
    s = rng.uniform(-1.0, 1.0, n)
    facet = rng.integers(0, 3, n)
    marker = rng.integers(1, 3, n)
    a_cell = np.stack([ref_kernels.a_cell(coords[t], D11[t], D22[t], D12[t], D[t], dt[t])
                       for t in range(n)])
    a_facet = np.stack([ref_kernels.a_facet(int(marker[t]), dt[t], r[t], coords[t], int(facet[t]))
                        for t in range(n)])
    L_cell = np.stack([ref_kernels.L_cell(coords[t], u0[t], dt[t], f[t]) for t in range(n)])
    L_facet = np.stack([ref_kernels.L_facet(int(marker[t]), dt[t], r[t], s[t], coords[t],
                                            int(facet[t])) for t in range(n)])
    flux = np.array([ref_kernels.flux_facet(coords[t], u0[t], int(facet[t])) for t in range(n)])
    np.savez_compressed(path, coords=coords, D11=D11, D22=D22, D12=D12, D=D, dt=dt, u0=u0, f=f,
                        r=r, s=s, facet=facet, marker=marker, a_cell=a_cell, a_facet=a_facet,
                        L_cell=L_cell, L_facet=L_facet, flux=flux)


def single_small_fixture(path):
    trap = wl.single_small(0)
    out = hsld.run_trap(trap, steps=100, snapshots=(1, 10, 100))
    mesh = out["oracles"][0].mesh
    nodes, w = hsld.point_weights(mesh, trap.cell_xy)
    snaps = {f"u_{n}": out["snapshots"][n][0] for n in (1, 10, 100)}
    cells = {f"c_{n}": np.sum(out["snapshots"][n][0][nodes] * w, axis=1) for n in (1, 10, 100)}
    np.savez_compressed(path, xy=trap.cell_xy, s=trap.cell_s, **snaps, **cells)


def odd_mesh_fixture(path):
    rng = np.random.Generator(np.random.PCG64(33))
    xy = np.stack([rng.uniform(0, 16.5, 9), rng.uniform(0, 3.5, 9)], 1)
    s = rng.lognormal(0, 0.5, 9)
    res = {"xy": xy, "s": s}
    for walls in (1, 0, 13):
        trap = wl.Trap(W=16.5, H=3.5, nx=33, ny=7, D=[49.0], g=[0.01], dt=0.1, steps=8,
                       walls=walls, cell_xy=xy, cell_s=s)
        out = hsld.run_trap(trap, steps=8)
        res[f"u_walls{walls}"] = out["u"][0]
        res[f"c_walls{walls}"] = out["cells"][0]
    np.savez_compressed(path, **res)


if __name__ == "__main__":
    element_fixture(os.path.join(HERE, "hsld_elements.npz"))
    single_small_fixture(os.path.join(HERE, "single_small_oracle.npz"))
    odd_mesh_fixture(os.path.join(HERE, "odd_mesh_oracle.npz"))
    print("fixtures written to", HERE)

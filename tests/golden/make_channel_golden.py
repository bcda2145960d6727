"""Generates tests/golden/channel_elements.npz: element tensors of the reference's own
flow-channel kernels (fenics/AdvectionDiffusion.h, compiled here from the reference
sources by oracle/ref_kernels.py) on seeded intervals and coefficients: the bilinear
cell tensor, the linear cell tensor, and both Robin end terms of each form.

Run from the repository root (needs the reference sources):
    python tests/golden/make_channel_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_kernels  # noqa: E402


def main(path=os.path.join(HERE, "channel_elements.npz")):
    if ref_kernels.build_if_available() is None:
        raise SystemExit("reference sources not found: cannot regenerate " + path)
    rng = np.random.Generator(np.random.PCG64(2025))
    n = 48
    x0 = rng.uniform(-5.0, 5.0, n)
    h = rng.uniform(0.05, 2.0, n)
    dt = rng.uniform(0.001, 0.2, n)
    D = rng.uniform(1.0, 3.0e4, n)
    v = rng.uniform(-60.0, 60.0, n)
    r = rng.uniform(0.0, 50.0, n)
    s = rng.uniform(-1.0, 1.0, n)
    u0 = rng.uniform(-1.0, 2.0, (n, 2))
    a_cell = np.zeros((n, 2, 2))
    L_cell = np.zeros((n, 2))
    a_facet = np.zeros((n, 2, 2, 2, 2))  # marker-1, facet, 2x2
    L_facet = np.zeros((n, 2, 2, 2))
    for t in range(n):
        c = [x0[t], x0[t] + h[t]]
        a_cell[t] = ref_kernels.adv_a_cell(c, dt[t], D[t], v[t])
        L_cell[t] = ref_kernels.adv_L_cell(c, u0[t], dt[t], D[t], v[t])
        for m in (1, 2):
            for f in (0, 1):
                a_facet[t, m - 1, f] = ref_kernels.adv_a_facet(m, dt[t], r[t], c, f)
                L_facet[t, m - 1, f] = ref_kernels.adv_L_facet(m, c, u0[t], dt[t], r[t], s[t], f)
    np.savez_compressed(path, x0=x0, h=h, dt=dt, D=D, v=v, r=r, s=s, u0=u0, a_cell=a_cell,
                        L_cell=L_cell, a_facet=a_facet, L_facet=L_facet)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()

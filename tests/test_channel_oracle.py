"""The wall-condition and flow-channel oracle (oracle/channel.py, oracle/hsld.py)
against the reference's own channel kernels (golden fixture made from
fenics/AdvectionDiffusion.h by tests/golden/make_channel_golden.py) and analytic known
answers.  CPU only."""
import os

import numpy as np
import pytest

from oracle import channel as chn
from oracle import hsld

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "channel_elements.npz")


def test_channel_elements_match_reference_kernels():
    z = np.load(GOLDEN)
    for t in range(len(z["h"])):
        h, dt, D, v = (float(z[k][t]) for k in ("h", "dt", "D", "v"))
        A = chn.element_a(h, dt, D, v)
        assert np.allclose(A, z["a_cell"][t], rtol=1e-13, atol=0), t
        b = chn.element_b(h, dt, D, v) @ z["u0"][t]
        assert np.allclose(b, z["L_cell"][t], rtol=1e-12, atol=1e-13 * np.abs(b).max()), t
        r, s = float(z["r"][t]), float(z["s"][t])
        for m in range(2):
            for f in range(2):
                e = np.zeros((2, 2))
                e[f, f] = 0.5 * dt * r  # the Robin end in the left side
                assert np.allclose(z["a_facet"][t, m, f], e, rtol=1e-14, atol=0)
                eb = np.zeros(2)
                eb[f] = -(0.5 * z["u0"][t][f] - s) * dt * r  # and in the right side
                assert np.allclose(z["L_facet"][t, m, f], eb, rtol=1e-14, atol=1e-300)


def test_channel_conserves_mass_without_flow_or_ends():
    ch = chn.Channel(W=20.0, nx=40, D=300.0, v=0.0, dt=0.1, substeps=5, r_left=0.0,
                     r_right=0.0)
    rng = np.random.default_rng(0)
    c = rng.uniform(0, 1, 41)
    h = 0.5
    w = np.full(41, h)
    w[[0, -1]] = h / 2  # 1^T M
    c1 = ch.step(c, np.zeros(41))
    assert abs(w @ c1 - w @ c) <= 1e-12 * (w @ c)
    # the flux goes in: nodal values raised by flux/L before each sub-step
    f = np.full(41, 0.3)
    c2 = ch.step(c, f)
    assert abs(w @ c2 - (w @ c + 0.3 * w.sum())) <= 1e-12 * (w @ c2)


def test_channel_flow_carries_mass_downstream():
    ch = chn.Channel(W=20.0, nx=80, D=1.0, v=30.0, dt=0.05, substeps=10, r_left=0.0,
                     r_right=30.0)
    x = np.linspace(0, 20, 81)
    c = np.exp(-((x - 5.0) ** 2))
    for _ in range(4):
        c = ch.step(c, np.zeros(81))
    assert abs(x[np.argmax(c)] - (5.0 + 30.0 * 0.2)) < 0.5


def test_robin_rates_as_the_reference_derives_them():
    rl, rr = chn.robin_rates(v=50.0, D=100.0, len_left=10.0, len_right=20.0)
    assert np.isclose(rl, 50.0 / (1 - np.exp(-5.0))) and np.isclose(rr, 50.0 / (np.exp(10.0) - 1))
    assert chn.robin_rates(0.0, 100.0, 10.0, 20.0) == (10.0, 5.0)


def test_dirichlet_values_hold_a_constant_state():
    """All walls at c = V and c = V inside: the discrete step keeps it (no decay)."""
    V = 2.5
    tr = chn.MicrofluidicTrap(10.0, 5.0, 20, 10, 490.0, 0.1, 0.0,
                              {s: (chn.DIRICHLET, V, 0.0) for s in range(4)})
    u = np.full(tr.mesh.n_nodes, V)
    u1 = tr.step(u)
    assert np.allclose(u1, V, rtol=1e-12)


def test_robin_steady_state_is_the_external_value():
    """Robin walls everywhere with external value s and no sources: c -> s."""
    tr = chn.MicrofluidicTrap(8.0, 4.0, 16, 8, 50.0, 1.0, 0.0,
                              {s: (chn.ROBIN, 1.5, 20.0) for s in range(4)})
    u = np.zeros(tr.mesh.n_nodes)
    for _ in range(200):
        u = tr.step(u)
    assert np.allclose(u, 1.5, rtol=1e-6)


def test_channel_walls_take_the_channel_values():
    tr = chn.MicrofluidicTrap(10.0, 5.0, 20, 10, 490.0, 0.1, 0.01,
                              {chn.BOTTOM: (chn.CHANNEL, 0, 0), chn.TOP: (chn.CHANNEL, 0, 0),
                               chn.LEFT: (chn.ROBIN, 0.0, 5.0), chn.RIGHT: (chn.ROBIN, 0.0, 5.0)},
                              channel={"velocity": 20.0, "D": 490.0, "rate": (5.0, 5.0),
                                       "substeps": 4, "well_scaling": 10.0})
    tr.channels[chn.BOTTOM][:] = np.linspace(0, 1, 21)
    F = hsld.point_load(tr.mesh, np.array([[5.0, 2.5]]), np.array([10.0]), scale=0.1)
    u = tr.step(np.zeros(tr.mesh.n_nodes), F)
    U = u.reshape(11, 21)
    assert np.allclose(U[0], np.linspace(0, 1, 21))
    assert np.allclose(U[10], 0.0)
    # the channels moved on: flux from the new field, then the sub-steps
    assert not np.allclose(tr.channels[chn.TOP], 0.0)

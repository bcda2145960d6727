"""The DOLFIN-free drop-in fHSL.h (eq_gb300/cpp/fHSL.h): class fenicsInterface with the
members Simulation reads and writes, driven the controller's way by
tests/cpp/shim_driver.cpp.

CPU: it compiles against the reference's own src/eQ.h (with its JSON library and a
stand-in mpi.h) and against the stand-in tests/cpp/eQ.h, and both decode the wall
conditions of eQ::data::parameters as createHSL does (src/fHSL.cpp:331-573),
including the reference's own boundaryCondition encoder.  GPU: the controller's
deposits through the DOF lookup table, a rotated tensor written into D11/D22/D12,
MICROFLUIDIC_TRAP walls with flow channels and DIRICHLET_UPDATE walls driven by
setBoundaryValues, each against the FP64 oracle."""
import math
import os
import subprocess

import numpy as np
import pytest

from eq_gb300 import build
from oracle import channel as chn
from oracle import hsld

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
REF_SRC = os.path.join(os.environ.get("EQ_REFERENCE_ROOT",
                                      os.path.join(os.path.dirname(ROOT), "reference")), "src")
STEPS = 6


def compile_driver(tmp_path, reference: bool):
    lib = build.build()
    exe = str(tmp_path / ("shim_ref" if reference else "shim_standin"))
    inc = ([os.path.join(CPP, "mpistub"), os.path.join(ROOT, "eq_gb300", "cpp"),
            os.path.join(ROOT, "include"), REF_SRC] if reference else
           [CPP, os.path.join(ROOT, "eq_gb300", "cpp"), os.path.join(ROOT, "include")])
    cmd = ["g++", "-std=c++17", "-O1"] + [f"-I{d}" for d in inc] + \
        [os.path.join(CPP, "shim_driver.cpp"), "-o", exe, "-L", os.path.dirname(lib),
         "-leqfield", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def parse_decode(text):
    out = {}
    for line in text.strip().splitlines():
        parts = line.split()
        walls = [tuple(float(x) for x in w.split(":")) for w in parts[1:5]]
        kv = dict(p.split("=") for p in parts[5:])
        out[parts[0]] = (walls, kv)
    return out


def robin_rates(v, D, lenl, lenr):
    if v > 1e-6:
        return v / (1.0 - math.exp(-lenl * v / D)), v / (math.exp(lenr * v / D) - 1.0)
    return D / lenl, D / lenr


def check_decode(d):
    # walls by side: bottom, top, left, right; kinds 0 Neumann, 1 Dirichlet, 2 Robin,
    # 3 channel, 4 well
    kinds = lambda name: [int(w[0]) for w in d[name][0]]  # noqa: E731
    assert kinds("NOWALLED") == [1, 1, 1, 1]
    assert kinds("THREEWALLED") == [1, 0, 0, 0]
    assert kinds("TWOWALLED") == [1, 1, 0, 0]
    assert kinds("ONEWALLED") == [1, 0, 1, 1]
    assert kinds("NEUMANN_3WALLED_TEST") == [1, 0, 1, 1]
    assert kinds("DIRICHLET_UPDATE") == [4, 4, 4, 4] and d["DIRICHLET_UPDATE"][1]["well"] == "1"
    rl, rr = robin_rates(40.0, 490.0, 10.0, 12.0)
    w, kv = d["MICROFLUIDIC_TRAP"]
    assert kinds("MICROFLUIDIC_TRAP") == [3, 3, 2, 2] and kv["ch"] == "1"
    assert w[2][2] == pytest.approx(rl, rel=1e-15) and w[3][2] == pytest.approx(rr, rel=1e-15)
    assert float(kv["sub"]) == 6 and float(kv["ws"]) == pytest.approx(62.5)
    assert float(kv["v"]) == 40.0 and float(kv["D"]) == 490.0
    w, kv = d["MICROFLUIDIC_VALUES"]
    assert kinds("MICROFLUIDIC_VALUES") == [1, 3, 1, 0]
    assert w[0][1] == pytest.approx(0.3) and w[2][1] == pytest.approx(0.7)
    w, kv = d["MICROFLUIDIC_NOFLOW"]
    assert float(kv["r"].split(",")[0]) == pytest.approx(490.0 / 10.0)
    # H-trap: Robin sides at the flow velocity, channels not stepped (walls at 0)
    w, kv = d["H_TRAP"]
    assert kinds("H_TRAP") == [1, 1, 2, 2] and w[2][2] == 40.0 and kv["ch"] == "0"


def test_drop_in_compiles_against_the_reference_eq_header_and_decodes_walls(tmp_path):
    if not os.path.exists(os.path.join(REF_SRC, "eQ.h")):
        pytest.skip("reference sources not present")
    exe = compile_driver(tmp_path, reference=True)
    r = subprocess.run([exe, "decode"], capture_output=True, text=True, check=True)
    d = parse_decode(r.stdout)
    check_decode(d)
    # the reference's own boundaryCondition encoder decodes like the hand encoding
    assert d["ENCODED"] == d["MICROFLUIDIC_TRAP"]
    # without a GPU the layer reports that no device is visible (with one, it steps)
    r = subprocess.run([exe, "aniso", str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 0 or (r.returncode == 3 and "init-error -4" in r.stdout), r.stdout


def test_drop_in_compiles_against_the_stand_in_and_decodes_walls(tmp_path):
    exe = compile_driver(tmp_path, reference=False)
    r = subprocess.run([exe, "decode"], capture_output=True, text=True, check=True)
    check_decode(parse_decode(r.stdout))


# ------------------------------------------------------------------------------- GPU
W, H, NPM, DT = 20.0, 10.0, 4.0, 0.1
NX, NY = int(W * NPM), int(H * NPM)
DEPOSITS = [((20, 30), lambda s: 1.0 + s), ((12, 61), lambda s: 0.5), ((33, 7), lambda s: 0.25 * s)]


def run_mode(tmp_path, mode):
    exe = compile_driver(tmp_path, reference=False)
    out = tmp_path / f"{mode}.bin"
    pvd = tmp_path / f"{mode}.pvd"
    r = subprocess.run([exe, mode, str(out), str(pvd)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    n = (NX + 1) * (NY + 1)
    raw = np.fromfile(out, dtype=np.float64).reshape(STEPS, n + 1 + 2 * (NX + 1))
    return raw[:, :n], raw[:, n], raw[:, n + 1:n + 2 + NX], raw[:, n + 2 + NX:], pvd


def deposit(u, s):
    u = u.copy()
    for (i, j), f in DEPOSITS:
        u[i * (NX + 1) + j] += f(s)
    return u


def rotated(turn):
    i, j = np.meshgrid(np.arange(NY + 1), np.arange(NX + 1), indexing="ij")
    th = turn + 0.6 * np.sin(2 * np.pi * j / NX) + 0.4 * i / NY
    c, s = np.cos(th), np.sin(th)
    return [(2.0 * c * c + 0.5 * s * s).ravel(), (2.0 * s * s + 0.5 * c * c).ravel(),
            (1.5 * s * c).ravel()]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.gpu
def test_drop_in_rotated_tensor_and_deposits_against_oracle(lib, tmp_path):
    fields, flux, _, _, pvd = run_mode(tmp_path, "aniso")
    u = np.zeros((NX + 1) * (NY + 1))
    o = None
    for s in range(STEPS):
        if s in (0, 3):
            t = rotated(0.0 if s == 0 else 0.9)
            o = hsld.HsldOracle(W, H, NX, NY, 49.0, DT, 0.0, hsld.WALL_BOTTOM, D11=t[0],
                                D22=t[1], D12=t[2])
        u = o.step(deposit(u, s))
        assert rel(fields[s], u) <= 1e-9, s
        assert flux[s] == pytest.approx(o.boundary_flux(u), rel=1e-9)
    text = pvd.read_text()
    assert text.count("<DataSet") == STEPS


@pytest.mark.gpu
def test_drop_in_microfluidic_walls_and_channels_against_oracle(lib, tmp_path):
    fields, flux, bottom, top, _ = run_mode(tmp_path, "microfluidic")
    rl, rr = robin_rates(40.0, 490.0, 10.0, 12.0)
    tr = chn.MicrofluidicTrap(W, H, NX, NY, 490.0, DT, 0.0,
                              {chn.BOTTOM: (chn.CHANNEL, 0.0, 0.0), chn.TOP: (chn.CHANNEL, 0.0, 0.0),
                               chn.LEFT: (chn.ROBIN, 0.0, rl), chn.RIGHT: (chn.ROBIN, 0.0, rr)},
                              {"velocity": 40.0, "D": 490.0, "rate": (rl, rr), "substeps": 6,
                               "well_scaling": 10.0 * 25.0 / NPM})
    u = np.zeros((NX + 1) * (NY + 1))
    for s in range(STEPS):
        u = tr.step(deposit(u, s))
        assert rel(fields[s], u) <= 1e-9, s
        assert rel(bottom[s], tr.channels[chn.BOTTOM]) <= 1e-9
        assert rel(top[s], tr.channels[chn.TOP]) <= 1e-9


@pytest.mark.gpu
def test_drop_in_dirichlet_update_walls_follow_set_boundary_values(lib, tmp_path):
    fields, _, _, _, _ = run_mode(tmp_path, "update")
    o = hsld.HsldOracle(W, H, NX, NY, 49.0, DT, 0.0, 15)
    u = np.zeros((NX + 1) * (NY + 1))
    for s in range(STEPS):
        dv = np.full(u.shape, 0.2 * (s + 1))
        u = o.step(deposit(u, s), None, dv)
        assert rel(fields[s], u) <= 1e-9, s

"""Output writers reading from a batch on the GPU (eqf_json_frame, eqf_vtk_write,
eqf_vtk_write_channel): what they write is the batch's state."""
import json
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from eq_gb300 import _lib
from eq_gb300 import field as F
from eq_gb300 import output
from eq_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_json_and_vtk_from_a_running_batch(lib, tmp_path):
    t = wl.scaled(wl.single_small(0), 64, 32, n_cells=60)
    tp = F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], 0)
    bc = wl.microfluidic_bc(wl.Trap(W=t.W, H=t.H, nx=t.nx, ny=t.ny, D=t.D, g=t.g, dt=t.dt,
                                    steps=1))
    with F.TrapBatch([tp, tp], F.default_opts(F.FP64)) as b:
        for k in range(2):
            b.set_boundaries(k, bc["walls"], bc["channel"])
            b.set_cells(k, t.cell_xy, t.cell_s * (k + 1))
        rec = output.JsonRecording(str(tmp_path / "run.json"), sim_number=1)
        series = output.VtkSeries(str(tmp_path / "hsl.pvd"))
        top = output.VtkSeries(str(tmp_path / "top.pvd"))
        ids = np.stack([np.arange(t.n_cells), np.zeros(t.n_cells, dtype=int)], 1)
        data = np.concatenate([t.cell_xy, np.zeros((t.n_cells, 3))], 1)
        for s in range(3):
            b.step(1)
            rec.frame(0.1 * (s + 1), batch=b, layers=[0, 1], ids=ids, data=data)
            series.write(b, 1, 0.1 * (s + 1))
            top.write_channel(b, 0, _lib.EQF_SIDE_TOP, 0.1 * (s + 1))
        u0, u1 = b.read_nodal(0), b.read_nodal(1)
        _, ch_top = b.read_channels(0)
        rec.close({"dt": t.dt})
        series.close()
        top.close()
    d = json.loads(open(tmp_path / "run.json").read())
    last = d["frames"][-1]
    assert np.array_equal(np.array(last["externalHSL"][0]), u0)
    assert np.array_equal(np.array(last["externalHSL"][1]), u1)
    assert len(last["cells"]) == t.n_cells
    root = ET.parse(tmp_path / "hsl000002.vtu").getroot()
    arr = [a for a in root.iter("DataArray") if a.get("Name") == "u"][0]
    assert np.array_equal(np.array(arr.text.split(), dtype=float), u1)
    root = ET.parse(tmp_path / "top000002.vtu").getroot()
    arr = [a for a in root.iter("DataArray") if a.get("Name") == "u"][0]
    assert np.array_equal(np.array(arr.text.split(), dtype=float), ch_top)

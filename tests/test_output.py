"""The reference's output formats (eqf_json_*, eqf_vtk_*): the JSON recording of
src/main.cpp:81-192 (v00_02) and the .pvd/.vtu snapshot series, written from host
fields.  CPU only (the writers are host code in the library)."""
import json
import math
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from eq_gb300 import output


@pytest.fixture
def lib():
    from eq_gb300 import _lib
    return _lib.load()


def test_json_recording_layout_and_values(lib, tmp_path):
    path = str(tmp_path / "rec.json")
    rng = np.random.Generator(np.random.PCG64(1))
    rec = output.JsonRecording(path, time_since_epoch=1700000000, node_id=0, sim_number=3)
    fields = rng.uniform(0, 10, (2, 21))
    ids = np.array([[7, 1], [9, 0]])
    data = np.array([[1.5, 2.25, 0.3, 3.1, 0.01, 12.0, 0.5],
                     [4.0, 1.0, math.pi, 2.0, 0.0, 1e-300, 7.0]])
    div = np.array([[0.1, 7, 3.9, 9, 2.0]])
    rec.frame(0.1, fields=fields, divisions=div, ids=ids, data=data)
    rec.frame(0.2, fields=fields * 2)
    rec.close({"dt": 0.1, "boundaryType": "MICROFLUIDIC_TRAP", "nodesPerMicronSignaling": 2})
    text = open(path).read()
    d = json.loads(text)
    # sorted keys, as the reference's JSON library writes objects
    assert list(d) == sorted(d)
    assert d["jsonSimVersion"] == "v00_02" and d["simNumber"] == 3
    assert d["timeSinceEpoch"] == 1700000000 and d["nodeID"] == 0
    assert d["cellDataFormat"] == [["id", "strainType"],
                                   ["x", "y", "angle", "length", "spring", "vargs"]]
    assert d["parameters"]["boundaryType"] == "MICROFLUIDIC_TRAP"
    f0, f1 = d["frames"]
    assert list(f0) == ["cells", "divisions", "externalHSL", "simTime"]
    assert f0["simTime"] == 0.1 and f1["simTime"] == 0.2
    assert f0["cells"][0] == [[7, 1], list(data[0])]
    assert f0["cells"][1][1][5] == 1e-300  # every value reads back exactly
    assert f0["divisions"] == [[0.1, 7, 3.9, 9, 2.0]]
    assert isinstance(f0["divisions"][0][1], int)
    assert np.array_equal(np.array(f0["externalHSL"]), fields)
    assert np.array_equal(np.array(f1["externalHSL"]), fields * 2)
    assert f1["cells"] == [] and f1["divisions"] == []
    assert '"spring","vargs"' in text and "2.0" in text  # integral doubles keep ".0"


def test_json_non_finite_values_are_null(lib, tmp_path):
    path = str(tmp_path / "nan.json")
    rec = output.JsonRecording(path)
    rec.frame(0.0, fields=np.array([[1.0, float("nan"), float("inf")]]))
    rec.close()
    d = json.loads(open(path).read())
    assert d["frames"][0]["externalHSL"] == [[1.0, None, None]]
    assert d["parameters"] == {}


def _vtu(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    arrays = {a.get("Name"): a for a in piece.iter("DataArray")}
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(-1, 3)
    u = np.array(arrays["u"].text.split(), dtype=float)
    conn = np.array(arrays["connectivity"].text.split(), dtype=int)
    types = np.array(arrays["types"].text.split(), dtype=int)
    return piece, pts, u, conn, types


def test_vtk_series_of_a_trap_and_a_channel(lib, tmp_path):
    pvd = str(tmp_path / "hsl.pvd")
    series = output.VtkSeries(pvd)
    nx, ny, W, H = 4, 3, 2.0, 1.5
    u = np.arange((nx + 1) * (ny + 1), dtype=float) * 0.1
    series.write_host(W, H, nx, ny, u, 0.0)
    series.write_host(W, H, nx, ny, u + 1, 0.5)
    series.close()
    coll = ET.parse(pvd).getroot()
    sets = coll.findall("Collection/DataSet")
    assert [s.get("file") for s in sets] == ["hsl000000.vtu", "hsl000001.vtu"]
    assert [float(s.get("timestep")) for s in sets] == [0.0, 0.5]
    piece, pts, uu, conn, types = _vtu(str(tmp_path / "hsl000001.vtu"))
    assert int(piece.get("NumberOfPoints")) == 20 and int(piece.get("NumberOfCells")) == 24
    assert np.array_equal(uu, u + 1)
    # vertex (i, j) at (j W/nx, i H/ny)
    assert np.allclose(pts[8], [3 * W / nx, 1 * H / ny, 0])  # node 8 = (1, 3)
    # square (0, 0): (v0, v1, v3) and (v0, v2, v3) with the cut (0,0)-(1,1)
    assert list(conn[:6]) == [0, 1, 6, 0, 5, 6]
    assert set(types) == {5}
    # a channel: nx + 1 nodes on [0, W] as line cells
    chan = output.VtkSeries(str(tmp_path / "top.pvd"))
    chan.write_host(W, 0.0, nx, 0, np.linspace(0, 1, nx + 1), 1.0)
    chan.close()
    piece, pts, uu, conn, types = _vtu(str(tmp_path / "top000000.vtu"))
    assert int(piece.get("NumberOfCells")) == nx and set(types) == {3}
    assert list(conn[:4]) == [0, 1, 1, 2] and np.allclose(pts[:, 1], 0)


def test_writer_argument_errors(lib, tmp_path):
    from eq_gb300 import _lib
    with pytest.raises(_lib.EqfError):
        output.VtkSeries(str(tmp_path / "no_extension"))
    with pytest.raises(_lib.EqfError):
        output.JsonRecording(str(tmp_path / "missing_dir" / "x.json"))

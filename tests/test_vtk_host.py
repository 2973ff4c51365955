"""VTK writer / reader (CPU): WriteVTK's encoding (appended raw, zlib blocks, UInt64 headers)
round trips exactly, vtk2trixi returns the reference reader's fields, collections list their
files."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("compress", [True, False])
def test_vtu_round_trip(pkg, tmp_path, nd, compress):
    vtk = pkg.vtk
    rng = np.random.default_rng(nd)
    n = 257
    pts = rng.normal(size=(n, nd))
    vel = rng.normal(size=(n, nd))
    rho = 1000 + rng.normal(size=n)
    p = rng.normal(size=n) * 1e4
    f = vtk.write_vtu(str(tmp_path / "fluid_1"), pts,
                      {"velocity": vel, "density": rho, "pressure": p,
                       "index": np.arange(1, n + 1), "particle_spacing": np.full(n, 0.02)},
                      {"time": 0.125, "ndims": nd}, compress=compress)
    root = ET.fromstring(_xml_head(f))
    assert root.get("type") == "UnstructuredGrid" and root.get("header_type") == "UInt64"
    assert (root.get("compressor") == "vtkZLibDataCompressor") == compress
    d = vtk.read_vtu(f)
    assert np.array_equal(d["points"][:, :nd], pts) and np.all(d["points"][:, nd:] == 0)
    assert np.array_equal(d["point_data"]["velocity"], vel)
    assert np.array_equal(d["point_data"]["density"], rho)
    assert np.array_equal(d["point_data"]["index"], np.arange(1, n + 1))
    t = vtk.vtk2trixi(f)
    assert t["time"] == 0.125 and t["particle_spacing"] == 0.02
    assert np.array_equal(t["coordinates"], pts) and np.array_equal(t["pressure"], p)


def _xml_head(f):
    buf = open(f, "rb").read()
    s = buf.index(b"<AppendedData")
    e = buf.rindex(b"</AppendedData>") + len(b"</AppendedData>")
    return buf[:s].decode() + "<AppendedData/>" + buf[e:].decode()


def test_vtk2trixi_defaults_and_pvd(pkg, tmp_path):
    vtk = pkg.vtk
    n = 5
    f = vtk.write_vtu(str(tmp_path / "x"), np.zeros((n, 2)), {"pressure": np.ones(n),
                                                             "my_quantity": np.arange(n) * 1.0},
                      {"ndims": 2})
    t = vtk.vtk2trixi(f)
    assert np.all(t["velocity"] == 0) and t["velocity"].shape == (n, 2)
    assert np.all(t["density"] == 0) and t["time"] == 0.0
    assert np.array_equal(t["my_quantity"], np.arange(n) * 1.0)
    pvd = vtk.write_pvd(str(tmp_path / "fluid_1"), [(0.0, "fluid_1_0.vtu"), (0.5, "fluid_1_1.vtu")])
    root = ET.parse(pvd).getroot()
    sets = root.findall("Collection/DataSet")
    assert [s.get("file") for s in sets] == ["fluid_1_0.vtu", "fluid_1_1.vtu"]
    assert float(sets[1].get("timestep")) == 0.5


def test_saving_callback_arguments(pkg):
    with pytest.raises(ValueError, match="ArgumentError"):
        pkg.SolutionSavingCallback(interval=2, dt=0.1)
    with pytest.raises(ValueError, match="ArgumentError"):
        pkg.SolutionSavingCallback()

"""VTK files written independently of the library's writer (tests/golden/make_vtu_fixtures.py
assembles them from the VTK XML format as WriteVTK.jl lays them out) read through vtk2trixi, and
the library's writer laid out like them.

The expectations restate the reference's vtk2trixi tests (test/io/read_vtk.jl): the standard
fields come back with their values and the particle order, a constant particle spacing as a
scalar, custom point and field data under their own names, `index` and `ndims` dropped, and a
velocity written as `initial_velocity` (trixi2vtk of an InitialCondition) found by substring
rather than a custom quantity whose name also contains "velocity" (:140-150)."""
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
SYSTEM_FILES = ["system_zlib_uint64.vtu", "system_raw_uint32.vtu", "system_base64_uint32.vtu",
                "system_ascii.vtu"]
N = 12


def _lattice():
    ix, iy = np.meshgrid(np.arange(4), np.arange(3), indexing="ij")
    return np.stack([0.1 * ix.ravel() + 1.0, 0.1 * iy.ravel() + 1.0], axis=1)


@pytest.mark.parametrize("name", SYSTEM_FILES)
def test_vtk2trixi_reads_fixture(pkg, name):
    t = pkg.vtk.vtk2trixi(str(GOLDEN / name))
    assert np.allclose(t["coordinates"], _lattice(), rtol=1e-15, atol=0)
    vel = np.column_stack([np.full(N, 2.0), -np.arange(N) * 0.5])
    assert np.array_equal(t["velocity"], vel)
    assert np.array_equal(t["density"], 1000.0 + np.arange(N))
    assert np.array_equal(t["pressure"], 900.0 - np.arange(N))
    assert t["particle_spacing"] == 0.1  # constant spacing -> scalar
    assert t["time"] == 0.25
    assert np.array_equal(t["my_custom_quantity"], np.full(N, 3.0))
    assert t["solver_version"] == "v0.4.1-fixture"
    assert "index" not in t and "ndims" not in t


def test_encodings_agree(pkg):
    ref = pkg.vtk.read_vtu(str(GOLDEN / SYSTEM_FILES[0]))
    for name in SYSTEM_FILES[1:]:
        d = pkg.vtk.read_vtu(str(GOLDEN / name))
        assert np.array_equal(d["points"], ref["points"])
        for k, v in ref["point_data"].items():
            assert np.array_equal(d["point_data"][k], v), (name, k)
            assert d["point_data"][k].dtype == v.dtype
        assert d["field_data"]["solver_version"] == ref["field_data"]["solver_version"]


def test_multi_block_compressed_array(pkg):
    """The pressure array of the default-encoding fixture is split into three zlib blocks."""
    buf = (GOLDEN / SYSTEM_FILES[0]).read_bytes()
    head = buf[:buf.index(b"<AppendedData")].decode()
    root = ET.fromstring(head + "</VTKFile>")  # the XML before the appended data
    off = int(next(e for e in root.iter("DataArray") if e.get("Name") == "pressure")
              .get("offset"))
    data = buf[buf.index(b"_", buf.index(b"<AppendedData")) + 1:]
    assert int.from_bytes(data[off:off + 8], "little") == 3
    assert np.array_equal(pkg.vtk.read_vtu(str(GOLDEN / SYSTEM_FILES[0]))["point_data"]
                          ["pressure"], 900.0 - np.arange(N))


def test_exact_field_match_rule(pkg):
    t = pkg.vtk.vtk2trixi(str(GOLDEN / "initial_condition_exact_match.vtu"))
    assert np.array_equal(t["velocity"], np.full((N, 2), 2.0))  # initial_velocity, not 42
    assert np.array_equal(t["center_of_mass_velocity"], np.full((N, 2), 42.0))
    assert np.array_equal(t["mass"], np.full(N, 10.0))
    assert np.all(t["density"] == 1000.0) and np.all(t["pressure"] == 900.0)
    assert t["time"] == 0.0  # no time field data: zero


def _layout(path):
    """Element paths and attributes of every DataArray except its offset and inline text."""
    buf = Path(path).read_bytes()
    if b"<AppendedData" in buf:
        s = buf.index(b"<AppendedData")
        e = buf.rindex(b"</AppendedData>") + len(b"</AppendedData>")
        buf = buf[:s] + buf[e:]
    root = ET.fromstring(buf.decode())
    out = [("root", tuple(sorted((k, v) for k, v in root.attrib.items())))]

    def walk(el, path):
        for ch in el:
            p = f"{path}/{ch.tag}"
            if ch.tag == "DataArray":
                attrs = {k: v for k, v in ch.attrib.items() if k != "offset"}
                if attrs.get("type") != "String":
                    attrs.pop("format", None)
                out.append((p, tuple(sorted(attrs.items()))))
            else:
                out.append((p, tuple(sorted((k, v) for k, v in ch.attrib.items()))))
                walk(ch, p)

    walk(root, "")
    return out


def test_writer_lays_files_out_like_the_fixture(pkg, tmp_path):
    """The library's writer, given the fixture's data, produces the same XML layout (elements,
    array names, types, components and tuple counts, header and compressor attributes)."""
    d = pkg.vtk.read_vtu(str(GOLDEN / SYSTEM_FILES[0]))
    pd = d["point_data"]
    f = pkg.vtk.write_vtu(str(tmp_path / "system"), d["points"][:, :2], pd,
                          {"time": 0.25, "ndims": 2, "solver_version": "v0.4.1-fixture"})
    assert _layout(f) == _layout(GOLDEN / SYSTEM_FILES[0])
    back = pkg.vtk.vtk2trixi(f)
    ref = pkg.vtk.vtk2trixi(str(GOLDEN / SYSTEM_FILES[0]))
    for k in ("coordinates", "velocity", "density", "pressure", "my_custom_quantity"):
        assert np.array_equal(back[k], ref[k]), k
    assert back["solver_version"] == ref["solver_version"]

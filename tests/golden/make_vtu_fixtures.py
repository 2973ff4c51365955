"""Write the .vtu fixtures of tests/test_vtk_fixtures.py, assembled byte by byte from the VTK XML
file format (UnstructuredGrid, "VTK File Formats", XML section) without the library's writer.

The files reproduce what the reference's trixi2vtk writes through WriteVTK.jl
(src/io/write_vtk.jl:120-215 for a system, 254-305 for an InitialCondition): vertex cells; point
data in the writer's order -- the system's fields, `index` (Int64, 1-based), `particle_spacing`,
custom quantities; field data `time`, `ndims` and the string `solver_version`; points always
with three components.  The values are those of the
reference's vtk2trixi tests (test/io/read_vtk.jl:3-13: 12 particles, velocity 2, density 1000,
pressure 900, particle spacing 0.1), on a 4 x 3 lattice instead of one repeated point so that
the particle order is checked too.  The files:

* system_zlib_uint64.vtu  -- WriteVTK's default: appended raw data, zlib blocks
  (vtkZLibDataCompressor), UInt64 headers; the pressure array split into three blocks;
* system_raw_uint32.vtu   -- appended raw data without compression, UInt32 headers;
* system_base64_uint32.vtu -- inline base64 ("binary") data, zlib blocks, UInt32 headers;
* system_ascii.vtu        -- inline ASCII data;
* initial_condition_exact_match.vtu -- trixi2vtk(::InitialCondition) with the custom quantity
  center_of_mass_velocity = 42 (test/io/read_vtk.jl:140-150): the velocity is written as
  `initial_velocity`, so vtk2trixi must take it by substring and not the custom quantity.

Run:  python tests/golden/make_vtu_fixtures.py   (rewrites the files next to this script)
"""
import base64
import struct
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
N = 12
TYPES = {"f8": "Float64", "i8": "Int64", "u1": "UInt8"}


def lattice():
    ix, iy = np.meshgrid(np.arange(4), np.arange(3), indexing="ij")
    return np.stack([0.1 * ix.ravel() + 1.0, 0.1 * iy.ravel() + 1.0])  # (2, 12), column order


def encode(arr, header, compress, block=None):
    """Data block of one array: [header][payload] with the header of the VTK XML format."""
    raw = np.ascontiguousarray(arr).astype(arr.dtype.newbyteorder("<")).tobytes()
    fmt = "<Q" if header == "UInt64" else "<I"
    if not compress:
        return struct.pack(fmt, len(raw)) + raw
    bs = block or max(len(raw), 1)
    chunks = [raw[k:k + bs] for k in range(0, len(raw), bs)] or [b""]
    comp = [zlib.compress(c) for c in chunks]
    last = len(chunks[-1])
    head = struct.pack(fmt[0] + fmt[1] * (3 + len(comp)), len(comp), bs, last,
                       *[len(c) for c in comp])
    return head + b"".join(comp)


def ascii_values(arr):
    return " ".join(repr(float(x)) if arr.dtype.kind == "f" else str(int(x))
                    for x in np.asarray(arr).ravel())


def string_ascii(s):
    """A vtkStringArray in ASCII: the bytes of each string as integers, each string closed by 0."""
    return " ".join(str(b) for b in s.encode()) + " 0"


def build(path, point_data, field_data, header="UInt64", compress=True, mode="appended",
          blocks=None):
    """point_data / field_data: list of (name, array, ncomp); strings only in field data."""
    points = np.zeros((N, 3))
    points[:, :2] = lattice().T
    arrays = []  # (section, name, vtk type, ncomp, ntuples, array)
    for name, a, k in field_data:
        arrays.append(("field", name, a, k))
    for name, a, k in point_data:
        arrays.append(("point", name, a, k))
    appended = b""
    xml_arrays = {"field": [], "point": [], "points": [], "cells": []}

    def data_array(section, name, a, k):
        nonlocal appended
        if isinstance(a, str):
            attrs = f'type="String" Name="{name}" NumberOfTuples="1" format="ascii"'
            xml_arrays[section].append(f"<DataArray {attrs}>{string_ascii(a)}</DataArray>")
            return
        vt = TYPES[a.dtype.str[1:]]
        comps = f' NumberOfComponents="{k}"' if k > 1 else ""
        tuples = f' NumberOfTuples="{a.size // k}"' if section == "field" else ""
        name_attr = f' Name="{name}"'
        if mode == "appended":
            blob = encode(a, header, compress, (blocks or {}).get(name))
            attrs = (f'type="{vt}"{name_attr}{comps}{tuples} format="appended" '
                     f'offset="{len(appended)}"')
            appended += blob
            xml_arrays[section].append(f"<DataArray {attrs}/>")
        elif mode == "binary":
            blob = encode(a, header, compress, (blocks or {}).get(name))
            if compress:  # compressed inline data: header and payload are encoded separately
                nb = struct.unpack_from("<Q" if header == "UInt64" else "<I", blob)[0]
                hlen = (3 + nb) * (8 if header == "UInt64" else 4)
                text = (base64.b64encode(blob[:hlen]) + base64.b64encode(blob[hlen:])).decode()
            else:
                text = base64.b64encode(blob).decode()
            attrs = f'type="{vt}"{name_attr}{comps}{tuples} format="binary"'
            xml_arrays[section].append(f"<DataArray {attrs}>{text}</DataArray>")
        else:
            attrs = f'type="{vt}"{name_attr}{comps}{tuples} format="ascii"'
            xml_arrays[section].append(f"<DataArray {attrs}>{ascii_values(a)}</DataArray>")

    for section, name, a, k in arrays:
        data_array(section, name, a, k)
    data_array("points", "Points", points, 3)
    data_array("cells", "connectivity", np.arange(N, dtype=np.int64), 1)
    data_array("cells", "offsets", np.arange(1, N + 1, dtype=np.int64), 1)
    data_array("cells", "types", np.ones(N, dtype=np.uint8), 1)
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    head = (f'<?xml version="1.0" encoding="utf-8"?>\n'
            f'<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
            f'header_type="{header}"{comp}>\n  <UnstructuredGrid>\n')
    body = "    <FieldData>\n" + "".join(f"      {x}\n" for x in xml_arrays["field"])
    body += "    </FieldData>\n"
    body += f'    <Piece NumberOfPoints="{N}" NumberOfCells="{N}">\n'
    body += "      <PointData>\n" + "".join(f"        {x}\n" for x in xml_arrays["point"])
    body += "      </PointData>\n"
    body += "      <Points>\n" + "".join(f"        {x}\n" for x in xml_arrays["points"])
    body += "      </Points>\n"
    body += "      <Cells>\n" + "".join(f"        {x}\n" for x in xml_arrays["cells"])
    body += "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n"
    out = head.encode() + body.encode()
    if mode == "appended":
        out += b'  <AppendedData encoding="raw">\n    _' + appended + b"\n  </AppendedData>\n"
    out += b"</VTKFile>\n"
    Path(path).write_bytes(out)


def system_fields():
    vel = np.full((N, 2), 2.0)
    vel[:, 1] = -np.arange(N) * 0.5  # distinct values: the component order is checked
    # the order of write_vtk.jl:178-198: the system's fields (write2vtk! of a fluid system),
    # index, particle_spacing, custom quantities
    point = [("velocity", vel, 2),
             ("density", np.full(N, 1000.0) + np.arange(N), 1),
             ("pressure", np.full(N, 900.0) - np.arange(N), 1),
             ("index", np.arange(1, N + 1, dtype=np.int64), 1),
             ("particle_spacing", np.full(N, 0.1), 1),
             ("my_custom_quantity", np.full(N, 3.0), 1)]
    field = [("time", np.array([0.25]), 1), ("ndims", np.array([2], dtype=np.int64), 1),
             ("solver_version", "v0.4.1-fixture", 1)]
    return point, field


def main():
    point, field = system_fields()
    build(HERE / "system_zlib_uint64.vtu", point, field, "UInt64", True, "appended",
          blocks={"pressure": 40})
    build(HERE / "system_raw_uint32.vtu", point, field, "UInt32", False, "appended")
    build(HERE / "system_base64_uint32.vtu", point, field, "UInt32", True, "binary")
    build(HERE / "system_ascii.vtu", point, field, "UInt64", False, "ascii")
    ic_point = [("index", np.arange(1, N + 1, dtype=np.int64), 1),
                ("particle_spacing", np.full(N, 0.1), 1),
                ("density", np.full(N, 1000.0), 1),
                ("initial_velocity", np.full((N, 2), 2.0), 2),
                ("mass", np.full(N, 10.0), 1),
                ("pressure", np.full(N, 900.0), 1),
                ("center_of_mass_velocity", np.full((N, 2), 42.0), 2)]
    ic_field = [("ndims", np.array([2], dtype=np.int64), 1)]
    build(HERE / "initial_condition_exact_match.vtu", ic_point, ic_field, "UInt64", True,
          "appended")


if __name__ == "__main__":
    main()

"""VTK output and restart: the on-disk format on either side of the path.

`trixi2vtk` writes the state of a Semidiscretization the way the reference's trixi2vtk does
(src/io/write_vtk.jl:127-215, 323-335, 487-500): one UnstructuredGrid file per system
("fluid_1", "boundary_1") with vertex cells, point data velocity / density / pressure (fluid),
hydrodynamic_density / pressure (wall), index (1-based) and particle_spacing, field data time and
ndims, optionally numbered per output with a ParaView collection (.pvd).  The encoding is the one
WriteVTK.jl produces by default -- XML, appended raw data, zlib-compressed blocks with UInt64
headers -- so that the reference's vtk2trixi / restart read these files and `vtk2trixi` here reads
the reference's.  `restart_from` restores v0 / u0 from such files (src/general/restart.jl:1-57;
fluid: velocity rows plus the density row, coordinates).  Snapshots are a device-to-host copy of
the state after a fresh system update (pressure of the current density, Adami wall state).
"""
from __future__ import annotations

import os
import struct
import xml.etree.ElementTree as ET
import zlib

import numpy as np

_VTK_TYPES = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32",
              np.dtype(np.int64): "Int64", np.dtype(np.int32): "Int32",
              np.dtype(np.uint8): "UInt8", np.dtype(np.uint32): "UInt32",
              np.dtype(np.uint64): "UInt64", np.dtype(np.int8): "Int8",
              np.dtype(np.int16): "Int16", np.dtype(np.uint16): "UInt16"}
_NP_TYPES = {v: k for k, v in _VTK_TYPES.items()}
VTK_VERTEX = 1
# the `solver_version` field data of the reference's files holds its git hash; ours names the
# library
SOLVER_VERSION = "trixiparticles.jl_gb300"


def _block(a: np.ndarray, compress: bool) -> bytes:
    raw = np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
    if not compress:
        return struct.pack("<Q", len(raw)) + raw
    c = zlib.compress(raw)
    # vtkZLibDataCompressor header (UInt64): blocks, block size, last block size, sizes
    return struct.pack("<QQQQ", 1, len(raw), len(raw), len(c)) + c


def write_vtu(filename: str, points: np.ndarray, point_data: dict, field_data: dict,
              compress: bool = True) -> str:
    """UnstructuredGrid of vertex cells at `points` (n, nd) with the given point / field data
    (numpy arrays; point data (n,) or (n, k)).  Returns the file name written."""
    pts = np.asarray(points, dtype=np.float64)
    n, nd = pts.shape
    p3 = np.zeros((n, 3))
    p3[:, :nd] = pts
    blobs, offset = [], 0

    def add(a):
        nonlocal offset
        b = _block(a, compress)
        blobs.append(b)
        off = offset
        offset += len(b)
        return off

    root = ET.Element("VTKFile", type="UnstructuredGrid", version="1.0",
                      byte_order="LittleEndian", header_type="UInt64")
    if compress:
        root.set("compressor", "vtkZLibDataCompressor")
    grid = ET.SubElement(root, "UnstructuredGrid")
    if field_data:
        fd = ET.SubElement(grid, "FieldData")
        for name, val in field_data.items():
            if isinstance(val, str):  # a vtkStringArray: byte values, closed by a 0, in ASCII
                ET.SubElement(fd, "DataArray", type="String", Name=name, NumberOfTuples="1",
                              format="ascii").text = " ".join(
                                  [str(b) for b in val.encode()] + ["0"])
                continue
            a = np.atleast_1d(np.asarray(val))
            if a.dtype.kind == "i":
                a = a.astype(np.int64)
            elif a.dtype.kind == "f":
                a = a.astype(np.float64)
            ET.SubElement(fd, "DataArray", type=_VTK_TYPES[a.dtype], Name=name,
                          NumberOfTuples=str(a.size), format="appended", offset=str(add(a)))
    piece = ET.SubElement(grid, "Piece", NumberOfPoints=str(n), NumberOfCells=str(n))
    pd = ET.SubElement(piece, "PointData")
    for name, val in point_data.items():
        a = np.asarray(val)
        if a.dtype.kind == "i":
            a = a.astype(np.int64)
        elif a.dtype.kind == "f":
            a = a.astype(np.float64)
        attrs = dict(type=_VTK_TYPES[a.dtype], Name=name, format="appended")
        if a.ndim == 2:
            attrs["NumberOfComponents"] = str(a.shape[1])
        attrs["offset"] = str(add(a))
        ET.SubElement(pd, "DataArray", **attrs)
    pe = ET.SubElement(piece, "Points")
    ET.SubElement(pe, "DataArray", type="Float64", Name="Points", NumberOfComponents="3",
                  format="appended", offset=str(add(p3)))
    ce = ET.SubElement(piece, "Cells")
    ET.SubElement(ce, "DataArray", type="Int64", Name="connectivity", format="appended",
                  offset=str(add(np.arange(n, dtype=np.int64))))
    ET.SubElement(ce, "DataArray", type="Int64", Name="offsets", format="appended",
                  offset=str(add(np.arange(1, n + 1, dtype=np.int64))))
    ET.SubElement(ce, "DataArray", type="UInt8", Name="types", format="appended",
                  offset=str(add(np.full(n, VTK_VERTEX, dtype=np.uint8))))
    ET.SubElement(root, "AppendedData", encoding="raw").text = "_"
    xml = ET.tostring(root, encoding="unicode")
    head, tail = xml.split('<AppendedData encoding="raw">_</AppendedData>')
    fn = filename if filename.endswith(".vtu") else filename + ".vtu"
    with open(fn, "wb") as f:
        f.write(b'<?xml version="1.0" encoding="utf-8"?>\n')
        f.write(head.encode())
        f.write(b'<AppendedData encoding="raw">\n_')
        for b in blobs:
            f.write(b)
        f.write(b"\n</AppendedData>")
        f.write(tail.encode())
    return fn


def _decode(buf: bytes, pos: int, dtype: np.dtype, compressed: bool,
            header: str = "UInt64") -> np.ndarray:
    """One data block at buf[pos:]: [UInt32|UInt64 header][payload]; compressed blocks carry the
    vtkZLibDataCompressor header (number of blocks, block size, last block size, sizes)."""
    f, w = ("<Q", 8) if header == "UInt64" else ("<I", 4)
    if compressed:
        (nb,) = struct.unpack_from(f, buf, pos)
        sizes = struct.unpack_from("<" + f[1] * nb, buf, pos + 3 * w)
        p = pos + (3 + nb) * w
        parts = []
        for s in sizes:
            parts.append(zlib.decompress(buf[p:p + s]))
            p += s
        raw = b"".join(parts)
    else:
        (nbytes,) = struct.unpack_from(f, buf, pos)
        raw = buf[pos + w:pos + w + nbytes]
    return np.frombuffer(raw, dtype=dtype.newbyteorder("<")).astype(dtype)


def _inline_binary(text: str, dtype: np.dtype, compressed: bool, header: str) -> np.ndarray:
    """format="binary": base64 text; a compressed array encodes its header and its payload as two
    separate base64 runs, an uncompressed one encodes [header][payload] as one."""
    import base64

    t = "".join(text.split())
    if not compressed:
        return _decode(base64.b64decode(t), 0, dtype, False, header)
    w = 8 if header == "UInt64" else 4
    f = "<Q" if w == 8 else "<I"
    # the header is 3 + nb words; its base64 run has ceil(bytes / 3) * 4 characters
    (nb,) = struct.unpack_from(f, base64.b64decode(t[:((w + 2) // 3) * 4])[:w])
    hbytes = (3 + nb) * w
    hchars = ((hbytes + 2) // 3) * 4
    head = base64.b64decode(t[:hchars])[:hbytes]
    payload = base64.b64decode(t[hchars:])
    return _decode(head + payload, 0, dtype, True, header)


def _string_ascii(text: str) -> str:
    """A vtkStringArray in ASCII: byte values, each string closed by a 0."""
    codes = [int(x) for x in text.split()]
    return bytes(c for c in codes if c != 0).decode()


def read_vtu(filename: str) -> dict:
    """Points, point data and field data of an UnstructuredGrid .vtu as WriteVTK.jl (and VTK)
    write them: appended raw data, inline base64 ("binary") or ASCII arrays, zlib-compressed or
    not, UInt32 or UInt64 headers; string arrays (ASCII) come back as str."""
    buf = open(filename, "rb").read()
    data = b""
    if b"<AppendedData" in buf:
        start = buf.index(b"<AppendedData")
        us = buf.index(b"_", start) + 1
        end = buf.rindex(b"</AppendedData>")
        data = buf[us:end]
        xml = (buf[:start].decode() + "<AppendedData/>"
               + buf[end + len(b"</AppendedData>"):].decode())
    else:
        xml = buf.decode()
    root = ET.fromstring(xml)
    if root.get("type") != "UnstructuredGrid":
        raise ValueError(f"{filename}: not an UnstructuredGrid file")
    if root.get("byte_order", "LittleEndian") != "LittleEndian":
        raise ValueError(f"{filename}: only little-endian files are supported")
    compressed = root.get("compressor") is not None
    header = root.get("header_type", "UInt32")
    if header not in ("UInt32", "UInt64"):
        raise ValueError(f"{filename}: unsupported header_type {header}")
    piece = root.find("UnstructuredGrid/Piece")
    n = int(piece.get("NumberOfPoints"))

    def arr(e):
        typ, fmt = e.get("type"), e.get("format", "ascii")
        if typ == "String":
            if fmt != "ascii":
                raise ValueError(f"{filename}: string arrays are read in ASCII only")
            return _string_ascii(e.text or "")
        dtype = _NP_TYPES[typ]
        if fmt == "appended":
            a = _decode(data, int(e.get("offset")), dtype, compressed, header)
        elif fmt == "binary":
            a = _inline_binary(e.text or "", dtype, compressed, header)
        elif fmt == "ascii":
            a = np.array((e.text or "").split(), dtype=np.float64).astype(dtype)
        else:
            raise ValueError(f"{filename}: unsupported DataArray format {fmt}")
        k = int(e.get("NumberOfComponents", "1"))
        return a.reshape(-1, k) if k > 1 else a

    out = {"points": arr(piece.find("Points/DataArray")).reshape(n, 3), "point_data": {},
           "field_data": {}}
    for e in piece.findall("PointData/DataArray"):
        out["point_data"][e.get("Name")] = arr(e)
    for e in root.findall("UnstructuredGrid/FieldData/DataArray"):
        out["field_data"][e.get("Name")] = arr(e)
    return out


def vtk2trixi(filename: str) -> dict:
    """The reference's vtk2trixi fields (src/io/read_vtk.jl:43-120): coordinates (n, ndims),
    velocity, density, pressure, particle_spacing (scalar when constant), time, plus the other
    point / field data; missing standard fields are zero."""
    d = read_vtu(filename)
    nd = int(np.atleast_1d(d["field_data"]["ndims"])[0])
    pdata = d["point_data"]
    coords = d["points"][:, :nd].copy()
    n = coords.shape[0]
    res = {}
    used = []
    for field in ("velocity", "density", "pressure", "particle_spacing"):
        key = field if field in pdata else next((k for k in pdata if field in k), None)
        if key is not None:
            res[field] = pdata[key]
            used.append(key)
        else:
            res[field] = np.zeros((n, nd)) if field == "velocity" else np.zeros(n)
    ps = res["particle_spacing"]
    res["particle_spacing"] = float(ps[0]) if np.all(ps == ps[0]) else ps
    res["coordinates"] = coords
    res["time"] = float(np.atleast_1d(d["field_data"].get("time", [0.0]))[0])
    for k, v in pdata.items():
        if k not in used and k not in ("index",):
            res[k] = v
    for k, v in d["field_data"].items():
        if k not in ("ndims", "time"):
            res[k] = v if isinstance(v, str) else (v[0] if np.size(v) == 1 else v)
    return res


def write_pvd(filename: str, entries) -> str:
    """ParaView collection of (time, file) entries."""
    root = ET.Element("VTKFile", type="Collection", version="1.0", byte_order="LittleEndian")
    col = ET.SubElement(root, "Collection")
    for t, f in entries:
        ET.SubElement(col, "DataSet", timestep=repr(float(t)), part="0", file=os.path.basename(f))
    fn = filename if filename.endswith(".pvd") else filename + ".pvd"
    with open(fn, "w") as fh:
        fh.write('<?xml version="1.0" encoding="utf-8"?>\n')
        fh.write(ET.tostring(root, encoding="unicode"))
    return fn


def snapshot(semi, v_ode, u_ode) -> dict:
    """Device-to-host copy of the state after a system update (pressure from the current
    density, Adami wall state): the arrays trixi2vtk writes."""
    import torch

    nd = semi.ndims
    dv = torch.empty_like(v_ode)
    from .semidiscretization import kick
    kick(dv, v_ode, u_ode, {"semi": semi}, 0.0)
    p_f = semi.fluid_pressure()
    p_w, rho_w, vol_w = semi.wall_state()
    semi.sync()
    v = v_ode.view(-1, nd + 1).cpu().numpy()
    return dict(u=u_ode.view(-1, nd).cpu().numpy(), velocity=v[:, :nd].copy(),
                density=v[:, nd].copy(), pressure=p_f.cpu().numpy(),
                wall_pressure=p_w.cpu().numpy(), wall_density=rho_w.cpu().numpy())


def trixi2vtk(semi, v_ode, u_ode, t: float, *, output_directory: str = "out", prefix: str = "",
              iter: int | None = None, collections: dict | None = None) -> list[str]:
    """Writes fluid_1 / boundary_1 files of the current state (write_vtk.jl:94-215)."""
    os.makedirs(output_directory, exist_ok=True)
    s = snapshot(semi, v_ode, u_ode)
    fl = semi.fluid.initial_condition
    wl = semi.wall.initial_condition
    pre = f"{prefix}_" if prefix else ""
    files = []
    for name, pts, pdata, spacing in (
            ("fluid_1", s["u"], {"velocity": s["velocity"], "density": s["density"],
                                 "pressure": s["pressure"]}, fl.particle_spacing),
            ("boundary_1", wl.coordinates, {"hydrodynamic_density": s["wall_density"],
                                            "pressure": s["wall_pressure"]},
             wl.particle_spacing)):
        base = os.path.join(output_directory, pre + name)
        fn = base + ("" if iter is None else f"_{iter}")
        n = pts.shape[0]
        pdata = dict(pdata)
        pdata["index"] = np.arange(1, n + 1, dtype=np.int64)
        pdata["particle_spacing"] = np.full(n, float(spacing))
        f = write_vtu(fn, pts, pdata, {"time": float(t), "ndims": int(semi.ndims),
                                       "solver_version": SOLVER_VERSION})
        files.append(f)
        if iter is not None and collections is not None:
            collections.setdefault(base, []).append((t, f))
            write_pvd(base, collections[base])
    return files


class SolutionSavingCallback:
    """SolutionSavingCallback(; interval or dt, output_directory, prefix): VTK snapshots during
    solve (src/callbacks/solution_saving.jl), at the start, every `interval` steps or every `dt`
    of integration time, and at the end."""

    def __init__(self, *, interval: int = -1, dt: float = 0.0, output_directory: str = "out",
                 prefix: str = "", save_initial_solution: bool = True,
                 save_final_solution: bool = True):
        if (interval > 0) == (dt > 0):
            raise ValueError("ArgumentError: set exactly one of `interval` and `dt`")
        self.interval = int(interval) if interval > 0 else None
        self.dt = float(dt) if dt > 0 else None
        self.output_directory = output_directory
        self.prefix = prefix
        self.save_initial_solution = save_initial_solution
        self.save_final_solution = save_final_solution
        self.files: list[str] = []
        self.collections: dict = {}
        self.count = 0
        self.last_t = None

    def save(self, semi, v, u, t):
        self.files += trixi2vtk(semi, v, u, t, output_directory=self.output_directory,
                                prefix=self.prefix, iter=self.count,
                                collections=self.collections)
        self.count += 1
        self.last_t = t


def restart_from(ode, semi, files) -> tuple:
    """set_initial_conditions! + time_span (restart.jl:1-57): v0 / u0 of the fluid from the
    fluid file (velocity rows and density row, coordinates); returns (ode, t_restart)."""
    import torch

    f_files = [f for f in files if "fluid" in os.path.basename(f)]
    if len(f_files) != 1:
        raise ValueError("ArgumentError: exactly one fluid restart file is expected")
    d = vtk2trixi(f_files[0])
    nd = semi.ndims
    n = d["coordinates"].shape[0]
    if n != semi.n_fluid:
        raise ValueError("ArgumentError: restart file particle count does not match the system")
    v = np.zeros((n, nd + 1))
    v[:, :nd] = d["velocity"]
    v[:, nd] = d["density"]
    ode.v0.copy_(torch.as_tensor(v.reshape(-1), device=ode.v0.device))
    ode.u0.copy_(torch.as_tensor(np.ascontiguousarray(d["coordinates"]).reshape(-1),
                                 device=ode.u0.device))
    t = d["time"]
    ode.tspan = (t, ode.tspan[1])
    return ode, t

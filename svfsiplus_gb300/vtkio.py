"""VTK XML files: the mesh input and result output of the reference (read_msh.cpp with
vtk_xml_parser.cpp; vtk_xml.cpp write_vtus), without the VTK library.

* ``read_vtk(path)`` reads .vtu (UnstructuredGrid) and .vtp (PolyData) files in the
  encodings VTK writes: ascii, inline base64 ("binary"), appended raw or base64, with
  UInt32 or UInt64 block headers, optionally zlib-compressed (vtkZLibDataCompressor).
* ``load_mesh(vtu, faces)`` builds the solver's mesh from a volume .vtu and face .vtp
  files the way the reference does: face node ids from the 1-based ``GlobalNodeID``
  point array (vtk_xml_parser.cpp:594-607), owner elements from the 1-based
  ``GlobalElementID`` cell array (:466-483).
* ``write_vtu(path, x, ien, fields)`` writes the result file through the library's
  ``svgpu_write_vtu`` (appended raw data); ``write_vtp`` writes face files for tests and
  for meshes made in code.
"""
from __future__ import annotations

import base64
import ctypes as C
import re
import struct
import xml.etree.ElementTree as ET
import zlib

import numpy as np

from . import mesh as _mesh

_DT = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "Int32": np.int32, "UInt64": np.uint64,
       "UInt32": np.uint32, "Int8": np.int8, "UInt8": np.uint8, "Int16": np.int16, "UInt16": np.uint16}


def _decode_block(raw: bytes, header: np.dtype, compressed: bool, dtype) -> np.ndarray:
    """One data array's bytes: a length header (or the zlib block table) then data."""
    hs = header.itemsize
    if not compressed:
        n = int(np.frombuffer(raw[:hs], dtype=header)[0])
        return np.frombuffer(raw[hs:hs + n], dtype=dtype)
    nb = int(np.frombuffer(raw[:hs], dtype=header)[0])
    tab = np.frombuffer(raw[hs:hs * (3 + nb)], dtype=header)
    csz = tab[2:2 + nb].astype(np.int64)
    pos = hs * (3 + nb)
    out = []
    for c in csz:
        out.append(zlib.decompress(raw[pos:pos + int(c)]))
        pos += int(c)
    return np.frombuffer(b"".join(out), dtype=dtype)


def _block_len(raw: bytes, header: np.dtype, compressed: bool) -> int:
    hs = header.itemsize
    if not compressed:
        return hs + int(np.frombuffer(raw[:hs], dtype=header)[0])
    nb = int(np.frombuffer(raw[:hs], dtype=header)[0])
    tab = np.frombuffer(raw[hs:hs * (3 + nb)], dtype=header)
    return hs * (3 + nb) + int(tab[2:2 + nb].astype(np.int64).sum())


def read_vtk(path) -> dict:
    """points (n,3), cells: connectivity/offsets/types (vtu) or polys (vtp), point_data
    and cell_data dicts of arrays (components as columns)."""
    data = open(path, "rb").read()
    i0 = data.find(b"<AppendedData")
    appended, enc = b"", "raw"
    if i0 >= 0:
        m = re.search(rb'<AppendedData[^>]*encoding="(\w+)"', data[i0:i0 + 200])
        enc = m.group(1).decode() if m else "raw"
        j = data.index(b"_", i0) + 1
        appended = data[j:data.rfind(b"</AppendedData>")]
        # AppendedData is VTKFile's last child: the part before it, closed, is the header
        root = ET.fromstring(data[:i0] + b"</VTKFile>")
    else:
        root = ET.fromstring(data)
    header = np.dtype(np.uint64 if root.get("header_type", "UInt32") == "UInt64" else np.uint32)
    compressed = root.get("compressor", "") != ""
    if root.get("byte_order", "LittleEndian") != "LittleEndian":
        raise ValueError("big-endian VTK files are not supported")
    if enc == "base64":
        appended = base64.b64decode(b"".join(appended.split()))

    def array(el):
        dt = _DT[el.get("type")]
        nc = int(el.get("NumberOfComponents", "1"))
        fmt = el.get("format", "ascii")
        if fmt == "ascii":
            a = np.array((el.text or "").split(), dtype=dt)
        elif fmt == "binary" and compressed:
            a = _decode_inline_compressed(el.text or "", header, dt)
        elif fmt == "binary":
            a = _decode_block(base64.b64decode("".join((el.text or "").split())), header, False, dt)
        elif fmt == "appended":
            blk = appended[int(el.get("offset")):]
            a = _decode_block(blk[:_block_len(blk, header, compressed)], header, compressed, dt)
        else:
            raise ValueError(f"unknown DataArray format {fmt}")
        return a.reshape(-1, nc) if nc > 1 else a

    piece = root.find(".//Piece")
    out = {"type": root.get("type"), "point_data": {}, "cell_data": {}}
    out["points"] = array(piece.find("Points/DataArray")).reshape(-1, 3).astype(np.float64)
    for el in piece.findall("PointData/DataArray"):
        out["point_data"][el.get("Name")] = array(el)
    for el in piece.findall("CellData/DataArray"):
        out["cell_data"][el.get("Name")] = array(el)
    for group in ("Cells", "Polys"):
        g = piece.find(group)
        if g is not None:
            out[group.lower()] = {el.get("Name"): array(el) for el in g.findall("DataArray")}
    return out


def _decode_inline_compressed(text: str, header: np.dtype, dt) -> np.ndarray:
    """Inline base64 with zlib: the block table is base64-encoded on its own, then the
    compressed blocks."""
    s = "".join(text.split())
    hs = header.itemsize
    # the table: nblocks, block size, last size, compressed sizes
    first = base64.b64decode(s[:4 * ((3 * hs + 2) // 3)])
    nb = int(np.frombuffer(first[:hs], dtype=header)[0])
    tl = 4 * (((3 + nb) * hs + 2) // 3)
    tab = np.frombuffer(base64.b64decode(s[:tl]), dtype=header)[:3 + nb]
    body = base64.b64decode(s[tl:])
    pos, parts = 0, []
    for c in tab[3:3 + nb].astype(np.int64):
        parts.append(zlib.decompress(body[pos:pos + int(c)]))
        pos += int(c)
    return np.frombuffer(b"".join(parts), dtype=dt)


def cell_connectivity(d: dict, npe: int) -> np.ndarray:
    """(nEl, npe) connectivity of a file whose cells all have npe nodes."""
    c = d.get("cells") or d.get("polys")
    conn, offs = np.asarray(c["connectivity"]).astype(np.int64), np.asarray(c["offsets"]).astype(np.int64)
    if not np.array_equal(np.diff(np.concatenate([[0], offs])), np.full(offs.size, npe)):
        raise ValueError(f"cells with other than {npe} nodes")
    return conn.reshape(-1, npe)


def load_mesh(vtu_path, face_paths: dict, domain_id: int | None = None) -> _mesh.PipeMesh:
    """The solver's mesh from a volume .vtu and face .vtp files (read_msh.cpp):
    coordinates and tets from the volume file; per face its triangles in global node
    ids (GlobalNodeID - 1), owner tets (GlobalElementID - 1) and sorted node list."""
    v = read_vtk(vtu_path)
    x = v["points"]
    ien = cell_connectivity(v, 4).astype(np.int32)
    faces = {}
    for name, p in face_paths.items():
        f = read_vtk(p)
        gid = np.asarray(f["point_data"]["GlobalNodeID"]).astype(np.int64) - 1
        eid = np.asarray(f["cell_data"]["GlobalElementID"]).astype(np.int64) - 1
        tri = gid[cell_connectivity(f, 3)].astype(np.int32)
        faces[name] = _mesh.Face(name, tri, eid.astype(np.int32), np.unique(tri).astype(np.int32))
    eid = None
    if domain_id is not None:
        eid = np.full(ien.shape[0], 1 << domain_id, dtype=np.int32)
    return _mesh.PipeMesh(x=x, ien=ien, faces=faces, radius=float(np.hypot(x[:, 0], x[:, 1]).max()),
                          length=float(np.ptp(x[:, 2])), inlet_profile=np.zeros(0), params={"source": str(vtu_path)},
                          eid=eid)


def write_vtu(path, x, ien, fields: dict | None = None):
    """Result file (svgpu_write_vtu): x (nNo,3), ien (nEl,4) or (nEl,3), fields of
    (nNo,) or (nNo, ncomp) arrays."""
    from .api import lib
    x = np.ascontiguousarray(x, dtype=np.float64)
    ien = np.ascontiguousarray(ien, dtype=np.int32)
    fields = fields or {}
    arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(x.shape[0], -1)) for a in fields.values()]
    n = len(arrs)
    names = (C.c_char_p * max(n, 1))(*[k.encode() for k in fields])
    ncomp = (C.c_int * max(n, 1))(*[a.shape[1] for a in arrs])
    data = (C.c_void_p * max(n, 1))(*[a.ctypes.data for a in arrs])
    rc = lib().svgpu_write_vtu(None, str(path).encode(), int(x.shape[0]), x.ctypes.data_as(C.c_void_p),
                               int(ien.shape[0]), int(ien.shape[1]), ien.ctypes.data_as(C.c_void_p), n, names, ncomp,
                               data)
    if rc != 0:
        raise RuntimeError(f"write_vtu failed ({rc}): {path}")


def write_vtp(path, points, tris, point_data=None, cell_data=None, encoding="appended", compress=False):
    """A PolyData face file in one of VTK's encodings ("ascii", "binary" inline base64,
    "appended" raw), optionally zlib-compressed, with UInt64 headers."""
    points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    tris = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    arrays = [("PointData", k, np.asarray(v)) for k, v in (point_data or {}).items()]
    arrays += [("CellData", k, np.asarray(v)) for k, v in (cell_data or {}).items()]
    arrays += [("Points", "Points", points), ("Polys", "connectivity", tris.ravel()),
               ("Polys", "offsets", np.arange(3, 3 * tris.shape[0] + 1, 3, dtype=np.int64))]
    rev = {np.dtype(v): k for k, v in _DT.items()}
    blocks, appended, off = {}, [], 0
    for grp, name, a in arrays:
        nc = a.shape[1] if a.ndim > 1 else 1
        raw = np.ascontiguousarray(a).tobytes()
        if compress:
            z = zlib.compress(raw)
            payload = struct.pack("<4Q", 1, len(raw), len(raw), len(z)) + z
        else:
            payload = struct.pack("<Q", len(raw)) + raw
        attrs = f'type="{rev[a.dtype]}" Name="{name}" NumberOfComponents="{nc}"'
        if encoding == "ascii":
            body = " ".join(str(v) for v in a.ravel())
            el = f'<DataArray {attrs} format="ascii">{body}</DataArray>'
        elif encoding == "binary":
            if compress:
                head = base64.b64encode(payload[:32]).decode()
                el = f'<DataArray {attrs} format="binary">{head}{base64.b64encode(payload[32:]).decode()}</DataArray>'
            else:
                el = f'<DataArray {attrs} format="binary">{base64.b64encode(payload).decode()}</DataArray>'
        else:
            el = f'<DataArray {attrs} format="appended" offset="{off}"/>'
            appended.append(payload)
            off += len(payload)
        blocks.setdefault(grp, []).append(el)
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    s = (f'<?xml version="1.0"?>\n<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" '
         f'header_type="UInt64"{comp}>\n<PolyData>\n<Piece NumberOfPoints="{points.shape[0]}" NumberOfPolys='
         f'"{tris.shape[0]}">\n')
    for grp in ("PointData", "CellData", "Points", "Polys"):
        s += f"<{grp}>\n" + "\n".join(blocks.get(grp, [])) + f"\n</{grp}>\n"
    s += "</Piece>\n</PolyData>\n"
    with open(path, "wb") as fh:
        fh.write(s.encode())
        if encoding == "appended":
            fh.write(b'<AppendedData encoding="raw">\n_' + b"".join(appended) + b"\n</AppendedData>\n")
        fh.write(b"</VTKFile>\n")


def write_mesh_files(directory, mesh: _mesh.PipeMesh, encoding="appended", compress=False):
    """The mesh as the reference's inputs: mesh-complete.mesh.vtu with GlobalNodeID /
    GlobalElementID (1-based) and one .vtp per face with the same ids."""
    import os
    os.makedirs(directory, exist_ok=True)
    vtu = os.path.join(directory, "mesh-complete.mesh.vtu")
    write_vtu(vtu, mesh.x, mesh.ien, {"GlobalNodeID": np.arange(1, mesh.nNo + 1, dtype=np.float64)})
    paths = {}
    for name, f in mesh.faces.items():
        nodes = f.gN
        local = np.searchsorted(nodes, f.ien)
        p = os.path.join(directory, f"{name}.vtp")
        write_vtp(p, mesh.x[nodes], local, point_data={"GlobalNodeID": (nodes + 1).astype(np.int32)},
                  cell_data={"GlobalElementID": (f.gE + 1).astype(np.int32)}, encoding=encoding, compress=compress)
        paths[name] = p
    return vtu, paths

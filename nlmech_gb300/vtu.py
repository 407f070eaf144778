"""VTU output and input in the layout of NLMech's simulation files.

model::Output (src/model/util.cpp:4-191) writes, per output step, a VTK XML
UnstructuredGrid through rw::writer::VtkWriter (src/rw/vtkWriter.cpp): the
points are the current positions x + u (appendNodes, vtkWriter.cpp:29-41),
the point data carry the tags the output deck asks for ("Displacement",
"Velocity", "Force" = force density times nodal volume, "Force_Density",
"Damage_Phi", "Damage_Z", "Fixity", "Node_Volume", ...) and the field data
the time ("TIME").  VTK stores the arrays "appended", base64-encoded and
zlib-compressed with a UInt32 block header; this module writes and reads
that encoding (VTK XML file-format documentation), so files go both ways
between this library and the reference's tools and ParaView.
"""
import base64
import re
import struct
import zlib

import numpy as np

_VTK_TYPE = {np.dtype("<f8"): "Float64", np.dtype("<f4"): "Float32",
             np.dtype("<i8"): "Int64", np.dtype("uint8"): "UInt8", np.dtype("<i4"): "Int32",
             np.dtype("<u8"): "UInt64"}
_NP_TYPE = {"Float64": "<f8", "Float32": "<f4", "Int64": "<i8", "UInt8": "u1", "Int32": "<i4",
            "UInt64": "<u8"}
_BLOCK = 1 << 15


def _encode(arr):
    raw = np.ascontiguousarray(arr).tobytes()
    blocks = [raw[k:k + _BLOCK] for k in range(0, len(raw), _BLOCK)] or [b""]
    comp = [zlib.compress(b) for b in blocks]
    last = len(raw) % _BLOCK  # size of a partial last block, 0 if it is full
    hdr = struct.pack("<%dI" % (3 + len(comp)), len(comp), _BLOCK, last,
                      *[len(c) for c in comp])
    return base64.b64encode(hdr).decode() + base64.b64encode(b"".join(comp)).decode()


def write_vtu(path, x, u=None, v=None, f=None, volume=None, phi=None, Z=None, fixity=None,
              time=None, extra=None):
    """Write one output step.  x, u, v, f: (n, 3) float64 in the caller's
    node order; f is the force density (written as "Force_Density" and,
    times the nodal volume, as "Force"); phi, Z: damage fields; fixity:
    uint8 bits per node; extra: {name: array} more point data."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
    pts = x + (np.asarray(u, dtype=np.float64).reshape(-1, 3) if u is not None else 0.)
    point_data = []
    if u is not None:
        point_data.append(("Displacement", np.asarray(u, dtype=np.float64).reshape(-1, 3)))
    if v is not None:
        point_data.append(("Velocity", np.asarray(v, dtype=np.float64).reshape(-1, 3)))
    if f is not None:
        fd = np.asarray(f, dtype=np.float64).reshape(-1, 3)
        if volume is not None:
            point_data.append(("Force", fd * np.asarray(volume, dtype=np.float64)[:, None]))
        point_data.append(("Force_Density", fd))
    if volume is not None:
        point_data.append(("Node_Volume", np.asarray(volume, dtype=np.float64)))
    if fixity is not None:
        point_data.append(("Fixity", np.asarray(fixity, dtype=np.uint8)))
    if phi is not None:
        point_data.append(("Damage_Phi", np.asarray(phi, dtype=np.float32)))
    if Z is not None:
        point_data.append(("Damage_Z", np.asarray(Z, dtype=np.float32)))
    for name, a in (extra or {}).items():
        point_data.append((name, np.asarray(a)))

    write_points(path, pts, point_data,
                 [] if time is None else [("TIME", np.array([time], dtype=np.float64))])


def write_points(path, points, point_data, field_data=()):
    """Write a VTU of vertex cells at points (n, 3) with point_data and
    field_data given as ordered [(name, array)] lists (model::Output's
    appendPointData / appendFieldData, in the caller's order)."""
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    chunks, off = [], [0]

    def add(arr):
        enc = _encode(arr)
        o = off[0]
        chunks.append(enc)
        off[0] += len(enc)
        return o

    def tag(name, arr, ntuples=None):
        a = np.asarray(arr)
        nc = a.shape[1] if a.ndim == 2 else 1
        typ = _VTK_TYPE[a.dtype.newbyteorder("<") if a.dtype.byteorder == ">" else a.dtype]
        extra_attr = ' NumberOfTuples="%d"' % ntuples if ntuples else ""
        return ('<DataArray type="%s" Name="%s" NumberOfComponents="%d"%s format="appended" '
                'offset="%d"/>' % (typ, name, nc, extra_attr, add(a)))

    lines = ['<?xml version="1.0"?>',
             '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
             'header_type="UInt32" compressor="vtkZLibDataCompressor">',
             '  <UnstructuredGrid>']
    if field_data:
        lines.append('    <FieldData>')
        lines += ['      ' + tag(name, np.atleast_1d(np.asarray(a, dtype=np.float64)),
                                 np.atleast_1d(a).size) for name, a in field_data]
        lines.append('    </FieldData>')
    lines.append('    <Piece NumberOfPoints="%d" NumberOfCells="%d">' % (n, n))
    lines.append('      <PointData>')
    lines += ['        ' + tag(name, a) for name, a in point_data]
    lines.append('      </PointData>')
    lines += ['      <Points>', '        ' + tag("Points", pts), '      </Points>']
    lines += ['      <Cells>',
              '        ' + tag("connectivity", np.arange(n, dtype=np.int64)),
              '        ' + tag("offsets", np.arange(1, n + 1, dtype=np.int64)),
              '        ' + tag("types", np.ones(n, dtype=np.uint8)),  # VTK_VERTEX
              '      </Cells>', '    </Piece>', '  </UnstructuredGrid>',
              '  <AppendedData encoding="base64">', '   _' + "".join(chunks),
              '  </AppendedData>', '</VTKFile>', '']
    with open(path, "w") as fh:
        fh.write("\n".join(lines))


def read_vtu(path):
    """All DataArrays of an appended, base64, zlib VTU file: {name: array}
    ((n, k) for k components, else (n,))."""
    txt = open(path, "rb").read().decode("latin1")
    app = txt[txt.index("<AppendedData"):]
    app = app[app.index("_") + 1:]
    app = app[:app.index("</AppendedData>")].strip()
    out = {}
    for attrs in re.findall(r"<DataArray([^>]*)>", txt):
        name = re.search(r'Name="([^"]*)"', attrs).group(1)
        typ = re.search(r'type="([^"]*)"', attrs).group(1)
        off = int(re.search(r'offset="\s*(\d+)', attrs).group(1))
        nc = re.search(r'NumberOfComponents="(\d+)"', attrs)
        nc = int(nc.group(1)) if nc else 1
        nb = struct.unpack("<I", base64.b64decode(app[off:off + 8])[:4])[0]
        hlen = 4 * (3 + nb)
        hchars = ((hlen + 2) // 3) * 4
        sizes = struct.unpack("<%dI" % (3 + nb), base64.b64decode(app[off:off + hchars])[:hlen])[3:]
        dchars = ((sum(sizes) + 2) // 3) * 4
        data = base64.b64decode(app[off + hchars:off + hchars + dchars])
        raw, p = b"", 0
        for sz in sizes:
            raw += zlib.decompress(data[p:p + sz])
            p += sz
        arr = np.frombuffer(raw, dtype=_NP_TYPE[typ])
        out[name] = arr.reshape(-1, nc) if nc > 1 else arr
    return out

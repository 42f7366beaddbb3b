"""Particle files in the classic Houdini BGEO format (version 5), as the reference's state
export and its initial fluid states use (PartioReaderWriter, extern/partio BGEO reader).

Layout (all big-endian): "Bgeo", "V", int32 version (5), nPoints, nPrims, nPointGroups,
nPrimGroups, nPointAttrib, nVertexAttrib, nPrimAttrib, nAttrib; then per point attribute a
uint16 name length, the name, uint16 component count, int32 type (0 float, 1 int,
5 vector, 4 indexed string followed by its string table) and one 32-bit default per
component; then per point the homogeneous position (4 floats) followed by the attributes'
32-bit components. Primitive and detail sections after the points are not read. gzip
files are read transparently.
"""
from __future__ import annotations

import gzip
import struct

import numpy as np

_FLOAT, _INT, _INDEXED, _VECTOR = 0, 1, 4, 5


def _open(path):
    with open(path, "rb") as f:
        head = f.read(2)
    return gzip.open(path, "rb") if head == b"\x1f\x8b" else open(path, "rb")


def read_bgeo(path):
    """Dict of attribute name -> array (n, components); "position" is (n, 3)."""
    with _open(path) as f:
        data = f.read()
    if data[:4] != b"Bgeo" or data[4:5] != b"V":
        raise ValueError(f"{path}: not a classic BGEO file")
    (version, n_points, n_prims, n_pgroups, n_prgroups, n_pattr, n_vattr, n_prattr,
     n_attr) = struct.unpack(">9i", data[5:41])
    if version != 5:
        raise ValueError(f"{path}: BGEO version {version}, expected 5")
    off = 41
    attrs = []  # (name, type, count)
    for _ in range(n_pattr):
        (nl,) = struct.unpack(">H", data[off:off + 2])
        off += 2
        name = data[off:off + nl].decode("ascii", "replace")
        off += nl
        count, typ = struct.unpack(">Hi", data[off:off + 6])
        off += 6
        if typ in (_FLOAT, _INT, _VECTOR):
            off += 4 * count  # defaults
        elif typ == _INDEXED:
            (ni,) = struct.unpack(">i", data[off:off + 4])
            off += 4
            for _ in range(ni):
                (sl,) = struct.unpack(">H", data[off:off + 2])
                off += 2 + sl
        else:
            raise ValueError(f"{path}: attribute {name!r} of unsupported type {typ}")
        attrs.append((name, typ, count))
    words = 4 + sum(c for _, _, c in attrs)
    nbytes = 4 * words * n_points
    if off + nbytes > len(data):
        raise ValueError(f"{path}: truncated point data")
    raw = np.frombuffer(data, dtype=">i4", count=words * n_points, offset=off).reshape(n_points, words)
    out = {"position": raw[:, 0:3].copy().view(">f4").astype(np.float32)}
    col = 4
    for name, typ, count in attrs:
        block = raw[:, col:col + count].copy()
        out[name] = block.view(">f4").astype(np.float32) if typ in (_FLOAT, _VECTOR) else block.astype(np.int32)
        col += count
    return out


def write_bgeo(path, position, **attributes):
    """Writes position (n, 3) and float (or int32) attributes (n,) or (n, k) uncompressed."""
    pos = np.asarray(position, dtype=np.float32).reshape(-1, 3)
    n = pos.shape[0]
    cols = [np.hstack([pos, np.ones((n, 1), np.float32)]).astype(">f4").view(">i4")]
    header_attrs = b""
    for name, val in attributes.items():
        a = np.asarray(val)
        a = a.reshape(n, -1)
        if np.issubdtype(a.dtype, np.integer):
            typ, block = _INT, a.astype(">i4")
        else:
            typ = _VECTOR if a.shape[1] == 3 else _FLOAT
            block = a.astype(">f4").view(">i4")
        nb = name.encode("ascii")
        header_attrs += struct.pack(">H", len(nb)) + nb + struct.pack(">Hi", a.shape[1], typ)
        header_attrs += b"\x00" * (4 * a.shape[1])
        cols.append(block)
    body = np.hstack(cols).astype(">i4").tobytes()
    head = b"Bgeo" + b"V" + struct.pack(">9i", 5, n, 0, 0, 0, len(attributes), 0, 0, 0)
    with open(path, "wb") as f:
        f.write(head + header_attrs + body)

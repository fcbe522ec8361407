"""ORACLE -- test infrastructure, not product code.

A numpy restatement of the Houdini classic binary geometry (.bgeo) point
layout that the reference writes through the partio library in
ExportBgeoFileCUDA (seepage_flows/include/kiri_utils.h:364-448) and reads
in ReadBgeoFileForGPU / ReadMultiBgeoFilesForGPU (kiri_utils.h:252-362).
Only tests/ use it, as the checker of sf_export_bgeo / sf_read_bgeo.

Pinned to partio: the reference vendors partio's sources
(extlib/include/partio; writeBGEO in io/BGEO.cpp), which oracle/build_ref.sh
compiles in place into oracle/_ref/libpartioref.so. This writer produces
partio's bytes for the reference's particle set (tests/test_bgeo_partio_cpu.py;
tests/golden/partio_export.npz carries partio's bytes for a seeded set), and
its reader and the library's agree with partio's reader. The layout, the
classic-bgeo (version 5) point layout as partio writes it:

  header, big-endian: int32 magic 'Bgeo', char 'V', int32 version 5, then
    int32 counts: points, primitives, point groups, primitive groups, point
    attributes (all but position), vertex attributes, primitive attributes,
    detail attributes
  per point attribute but position: uint16 name length, name bytes, uint16
    component count, int32 type (0 float, 1 int, 5 vector; 4 indexed string,
    followed by int32 string count and uint16-length strings), then one
    int32 default per component (0)
  per point: float32 x, y, z, w = 1, then each attribute's components, all
    big-endian 4-byte words
  end: the bytes 0x00, 0xff

The reference exports the attributes position (vector 3), Cd (float 3),
pscale (float 1) and label (int 1), in its particles' current order.
"""

from __future__ import annotations

import struct

import numpy as np

MAGIC = (ord("B") << 24) | (ord("g") << 16) | (ord("e") << 8) | ord("o")
TYPE_FLOAT, TYPE_INT, TYPE_INDEX, TYPE_VECTOR = 0, 1, 4, 5

# the reference's export attributes after position: (name, components, type)
EXPORT_ATTRS = (("Cd", 3, TYPE_FLOAT), ("pscale", 1, TYPE_FLOAT), ("label", 1, TYPE_INT))


def header(n: int, attrs=EXPORT_ATTRS) -> bytes:
    out = bytearray(struct.pack(">icii", MAGIC, b"V", 5, n))
    out += struct.pack(">7i", 0, 0, 0, len(attrs), 0, 0, 0)
    for name, count, typ in attrs:
        nb = name.encode()
        out += struct.pack(">H", len(nb)) + nb + struct.pack(">Hi", count, typ) + b"\0" * (4 * count)
    return bytes(out)


TRAILER = b"\x00\xff"


def records(pos: np.ndarray, col: np.ndarray, radius: np.ndarray, label: np.ndarray) -> bytes:
    """The point records: position with w = 1, Cd, pscale, label."""
    n = len(pos)
    rec = np.empty((n, 9), dtype=">u4")
    f = rec.view(">f4")
    f[:, 0:3] = np.asarray(pos, np.float32).reshape(n, 3)
    f[:, 3] = 1.0
    f[:, 4:7] = np.asarray(col, np.float32).reshape(n, 3)
    f[:, 7] = np.asarray(radius, np.float32).reshape(n)
    rec[:, 8] = np.asarray(label).astype(np.int64).astype(np.int32).view(np.uint32)
    return rec.tobytes()


def write_bytes(pos, col, radius, label) -> bytes:
    """The whole file ExportBgeoFileCUDA writes for these arrays."""
    return header(len(pos)) + records(pos, col, radius, label) + TRAILER


def read(data: bytes) -> dict:
    """Point attributes of a classic .bgeo (float, int, vector and indexed-string
    attributes; the position's w is dropped, as partio's reader does)."""
    magic, vchar, version, n = struct.unpack_from(">icii", data, 0)
    if magic != MAGIC or vchar != b"V" or version != 5:
        raise ValueError("not a version-5 classic bgeo")
    o = 13
    counts = struct.unpack_from(">7i", data, o)
    o += 28
    n_attr = counts[3]
    attrs = []
    for _ in range(n_attr):
        (ln,) = struct.unpack_from(">H", data, o)
        o += 2
        name = data[o:o + ln].decode()
        o += ln
        count, typ = struct.unpack_from(">Hi", data, o)
        o += 6
        if typ == TYPE_INDEX:
            (ns,) = struct.unpack_from(">i", data, o)
            o += 4
            for _ in range(ns):
                (sl,) = struct.unpack_from(">H", data, o)
                o += 2 + sl
        else:
            o += 4 * count
        attrs.append((name, count, typ))
    width = 4 + sum(c for _, c, _ in attrs)
    words = np.frombuffer(data, dtype=">u4", count=n * width, offset=o).reshape(n, width)
    out = {"position": words[:, 0:3].view(">f4").astype(np.float32)}
    k = 4
    for name, count, typ in attrs:
        block = words[:, k:k + count]
        if typ in (TYPE_FLOAT, TYPE_VECTOR):
            out[name] = block.view(">f4").astype(np.float32)
        else:
            out[name] = block.view(">i4").astype(np.int32)
        k += count
    return out


def read_for_gpu(data: bytes, flip_yz: bool = False) -> np.ndarray:
    """ReadBgeoFileForGPU: (x, y, z, pscale) per point, pscale 0.01 when the
    file has none, y and z swapped when flip_yz."""
    a = read(data)
    p = a["position"]
    s = a["pscale"][:, 0] if "pscale" in a else np.full(len(p), 0.01, np.float32)
    out = np.empty((len(p), 4), np.float32)
    out[:, 0] = p[:, 0]
    out[:, 1] = p[:, 2] if flip_yz else p[:, 1]
    out[:, 2] = p[:, 1] if flip_yz else p[:, 2]
    out[:, 3] = s
    return out

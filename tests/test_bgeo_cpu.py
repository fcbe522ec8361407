"""The .bgeo format (CPU): the oracle's writer against hand-built bytes, its
reader round trip, and the library's host-side reader (sf_read_bgeo, which
needs no GPU) on files the oracle wrote: positions, pscale, the y/z flip,
files without pscale, skipped indexed-string attributes and malformed files."""

import struct

import numpy as np
import pytest

from oracle import bgeo
from sph_seepage_flows_gb300 import build, capi


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return capi.load()


def test_export_header_bytes_by_hand():
    """Two points: magic, version, counts, then the Cd / pscale / label
    definitions with zero defaults (98 bytes), 36 bytes per point, 0x00 0xff."""
    want = b"Bgeo" + b"V" + struct.pack(">i", 5) + struct.pack(">8i", 2, 0, 0, 0, 3, 0, 0, 0)
    want += struct.pack(">H", 2) + b"Cd" + struct.pack(">Hi", 3, 0) + b"\0" * 12
    want += struct.pack(">H", 6) + b"pscale" + struct.pack(">Hi", 1, 0) + b"\0" * 4
    want += struct.pack(">H", 5) + b"label" + struct.pack(">Hi", 1, 1) + b"\0" * 4
    assert len(want) == 98
    assert bgeo.header(2) == want
    rec = bgeo.records(np.array([[1.0, 2.0, 3.0], [0, 0, 0]]), np.array([[0.5, 0.25, 1.0], [0, 0, 0]]),
                       np.array([0.01, 0.02]), np.array([1, 0]))
    assert rec[:36] == struct.pack(">8fi", 1.0, 2.0, 3.0, 1.0, 0.5, 0.25, 1.0, np.float32(0.01), 1)
    assert len(bgeo.write_bytes(np.zeros((2, 3)), np.zeros((2, 3)), np.zeros(2), np.zeros(2))) == 98 + 72 + 2


def sample(n, seed=0):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, 3)).astype(np.float32), rng.random((n, 3)).astype(np.float32),
            rng.random(n).astype(np.float32) * 0.01, rng.integers(0, 2, n))


def test_oracle_round_trip():
    pos, col, rad, lab = sample(257)
    a = bgeo.read(bgeo.write_bytes(pos, col, rad, lab))
    assert np.array_equal(a["position"], pos) and np.array_equal(a["Cd"], col)
    assert np.array_equal(a["pscale"][:, 0], rad) and np.array_equal(a["label"][:, 0], lab)


@pytest.mark.parametrize("flip", [False, True])
def test_library_reader_matches_oracle(lib, tmp_path, flip):
    pos, col, rad, lab = sample(1000, 3)
    f = tmp_path / "s.bgeo"
    f.write_bytes(bgeo.write_bytes(pos, col, rad, lab))
    got = capi.read_bgeo(str(f), flip)
    assert np.array_equal(got, bgeo.read_for_gpu(f.read_bytes(), flip))
    assert np.array_equal(got[:, 3], rad)


def test_reader_without_pscale_and_with_string_attribute(lib, tmp_path):
    """pscale 0.01 when absent; an indexed-string attribute's table is skipped."""
    n = 5
    attrs = (("name", 1, bgeo.TYPE_INDEX), ("v", 3, bgeo.TYPE_VECTOR), ("pscale", 1, bgeo.TYPE_FLOAT))
    head = bytearray(struct.pack(">icii", bgeo.MAGIC, b"V", 5, n) + struct.pack(">7i", 0, 0, 0, 3, 0, 0, 0))
    head += struct.pack(">H", 4) + b"name" + struct.pack(">Hi", 1, 4) + struct.pack(">i", 2)
    head += struct.pack(">H", 3) + b"abc" + struct.pack(">H", 1) + b"z"
    head += struct.pack(">H", 1) + b"v" + struct.pack(">Hi", 3, 5) + b"\0" * 12
    head += struct.pack(">H", 6) + b"pscale" + struct.pack(">Hi", 1, 0) + b"\0" * 4
    rows = b"".join(struct.pack(">4f", i, 2 * i, 3 * i, 1) + struct.pack(">i", i % 2) +
                    struct.pack(">3f", 0, 0, 0) + struct.pack(">f", 0.5 + i) for i in range(n))
    f = tmp_path / "s.bgeo"
    f.write_bytes(bytes(head) + rows + bgeo.TRAILER)
    got = capi.read_bgeo(str(f))
    assert np.array_equal(got[:, :3], np.array([[i, 2 * i, 3 * i] for i in range(n)], np.float32))
    assert np.array_equal(got[:, 3], 0.5 + np.arange(n, dtype=np.float32))
    # no pscale at all
    g = tmp_path / "t.bgeo"
    g.write_bytes(bgeo.header(n, (("Cd", 3, bgeo.TYPE_FLOAT),)) +
                  b"".join(struct.pack(">7f", i, i, i, 1, 0, 0, 0) for i in range(n)) + bgeo.TRAILER)
    got = capi.read_bgeo(str(g))
    assert np.array_equal(got[:, 3], np.full(n, 0.01, np.float32))
    assert np.array_equal(got, bgeo.read_for_gpu(g.read_bytes()))


def test_reader_rejects_malformed_files(lib, tmp_path):
    pos, col, rad, lab = sample(10)
    good = bgeo.write_bytes(pos, col, rad, lab)
    for name, data in (("magic", b"Xgeo" + good[4:]), ("version", good[:5] + struct.pack(">i", 4) + good[9:]),
                       ("short", good[:60]), ("points", good[:98 + 36 * 5])):
        f = tmp_path / f"{name}.bgeo"
        f.write_bytes(data)
        with pytest.raises(RuntimeError, match="sf_read_bgeo"):
            capi.read_bgeo(str(f))
    with pytest.raises(RuntimeError, match="open"):
        capi.read_bgeo(str(tmp_path / "missing.bgeo"))
    # the point count alone, and a capacity that is too small
    f = tmp_path / "ok.bgeo"
    f.write_bytes(good)
    n = capi.ctypes.c_int64()
    assert lib.sf_read_bgeo(str(f).encode(), 0, None, 0, capi.ctypes.byref(n)) == 0 and n.value == 10
    buf = np.zeros((9, 4), np.float32)
    assert lib.sf_read_bgeo(str(f).encode(), 0, capi._fptr(buf), 9, capi.ctypes.byref(n)) == 1

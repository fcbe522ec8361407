"""The .bgeo format pinned to partio, the library the reference writes and
reads it with (ExportBgeoFileCUDA / ReadBgeoFileForGPU, seepage_flows/
include/kiri_utils.h:252-448). partio's own writer and reader are compiled
from the copy the reference vendors (extlib/include/partio) by
oracle/build_ref.sh where the reference sources are mounted; the committed
fixture tests/golden/partio_export.npz (tests/golden/make_partio_golden.py)
carries partio's bytes for a seeded 300-point set to places without them.

Checks: the format oracle (oracle/bgeo.py) writes partio's bytes; the
library's host-side reader (sf_read_bgeo, no GPU) reads partio's file as
partio's reader does; where partio is built, random point sets of several
sizes go both ways.
"""

import numpy as np
import pytest

from helpers import load_golden
from oracle import bgeo
from sph_seepage_flows_gb300 import build, capi


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return capi.load()


@pytest.fixture(scope="module")
def partio():
    import oracle
    oracle.build_ref()
    if oracle.partio_lib() is None:
        pytest.skip("partio harness needs the reference sources (oracle/build_ref.sh)")
    return oracle


def test_oracle_writes_partio_bytes():
    g = load_golden("partio_export.npz")
    assert bgeo.write_bytes(g["pos"], g["col"], g["radius"], g["label"]) == g["bgeo"].tobytes()


@pytest.mark.parametrize("flip", [False, True])
def test_library_reader_reads_partio_file(lib, tmp_path, flip):
    g = load_golden("partio_export.npz")
    f = tmp_path / "p.bgeo"
    f.write_bytes(g["bgeo"].tobytes())
    got = capi.read_bgeo(str(f), flip)
    want = g["pos"][:, [0, 2, 1]] if flip else g["pos"]
    assert np.array_equal(got[:, :3], want)
    assert np.array_equal(got[:, 3], g["radius"])


@pytest.mark.parametrize("n", [0, 1, 17, 1000])
def test_partio_and_oracle_agree_both_ways(partio, lib, tmp_path, n):
    rng = np.random.default_rng(n + 5)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    col = rng.random((n, 3)).astype(np.float32)
    rad = (rng.random(n) * 0.02).astype(np.float32)
    lab = rng.integers(0, 2, n).astype(np.int64)
    f = tmp_path / f"partio{n}.bgeo"
    partio.partio_write(f, pos, col, rad, lab)
    assert f.read_bytes() == bgeo.write_bytes(pos, col, rad, lab)
    g = tmp_path / f"ours{n}.bgeo"
    g.write_bytes(bgeo.write_bytes(pos, col, rad, lab))
    for flip in (False, True):
        want = partio.partio_read_for_gpu(g, flip)
        assert np.array_equal(want, bgeo.read_for_gpu(g.read_bytes(), flip))
        if n:
            assert np.array_equal(capi.read_bgeo(str(f), flip), want)


def test_library_reader_matches_partio_without_pscale(partio, lib, tmp_path):
    """A file with position and Cd only: both readers supply pscale 0.01."""
    n = 9
    f = tmp_path / "nopscale.bgeo"
    f.write_bytes(bgeo.header(n, (("Cd", 3, bgeo.TYPE_FLOAT),)) +
                  b"".join(np.array([i, 2 * i, -i, 1, 0, 0, 0], ">f4").tobytes() for i in range(n)) + bgeo.TRAILER)
    assert np.array_equal(capi.read_bgeo(str(f)), partio.partio_read_for_gpu(f))

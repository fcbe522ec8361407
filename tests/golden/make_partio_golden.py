"""Writes tests/golden/partio_export.npz: a seeded particle set and the .bgeo
bytes partio's own writer produces for it, built the way the reference's
ExportBgeoFileCUDA builds its particle set (seepage_flows/include/
kiri_utils.h:364-448; partio compiled from the reference's vendored sources by
oracle/build_ref.sh). The GPU tests compare the library's export with these
bytes where the reference sources (and so partio) are not available.

    python tests/golden/make_partio_golden.py
"""

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def particle_set(n=300, seed=31):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1.0, 2.0, (n, 3)).astype(np.float32)
    col = rng.random((n, 3)).astype(np.float32)
    rad = rng.choice(np.array([0.005, 0.01], np.float32), n)
    lab = rng.integers(0, 2, n).astype(np.int64)
    return pos, col, rad, lab


def main():
    oracle.build_ref()
    if oracle.partio_lib() is None:
        raise SystemExit("partio harness not built: the reference sources are needed")
    pos, col, rad, lab = particle_set()
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "p.bgeo")
        oracle.partio_write(f, pos, col, rad, lab)
        data = open(f, "rb").read()
    np.savez_compressed(os.path.join(HERE, "partio_export.npz"), pos=pos, col=col, radius=rad, label=lab,
                        bgeo=np.frombuffer(data, np.uint8))
    print("wrote partio_export.npz:", len(data), "bytes of .bgeo for", len(rad), "points")


if __name__ == "__main__":
    main()

"""Host-side parts of the C++ facade (include/sf_kiri_facade.hpp) against the
reference emitters' output (tests/golden/emitters.npz): world-boundary shell
and square / circle / rectangle emitter samples. Compiled with g++ against
the CUDA headers only; runs without a GPU."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    out = str(tmp_path_factory.mktemp("facade") / "emitter_points")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", f"{cuda}/include",
                    os.path.join(ROOT, "tests", "cpp", "emitter_points.cpp"), "-o", out], check=True)
    return out


def run(exe, *args):
    r = subprocess.run([exe, *map(str, args)], capture_output=True, check=True)
    return np.frombuffer(r.stdout, dtype=np.float32).reshape(-1, 3)


def test_world_boundary_matches_reference(exe):
    g = load_golden("emitters.npz")
    pos = run(exe, "world", 0.0, 0.0, 0.0, 0.4, 0.4, 0.4, 0.01)
    assert np.array_equal(pos, g["world_boundary_small"])
    big = run(exe, "world", 0.0, 0.0, 0.0, 4.0, 0.6, 1.0, 0.005)
    assert big.shape[0] == int(g["world_boundary_large_count"])


@pytest.mark.parametrize("kind,name,a,b", [(0, "square", 0.05, 0.0), (1, "circle", 0.17, 0.0),
                                           (2, "rectangle", 0.22, 0.18)])
def test_emitter_samples_match_reference(exe, kind, name, a, b):
    g = load_golden("emitters.npz")
    pts = run(exe, "emit", kind, 0.01, a, b)
    assert np.array_equal(pts, g["emit_" + name]), (pts.shape, g["emit_" + name].shape)

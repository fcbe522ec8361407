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


@pytest.fixture(scope="module")
def shape_exe(tmp_path_factory):
    """tests/cpp/shape_import.cpp linked against libsf_gb300.so (for the .bgeo
    reader), with DB_PBR_PATH at a temporary asset root holding the seeded
    stand-in shape of tests/golden/shapes.npz as bgeo/shapes/ball.bgeo."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from oracle import bgeo
    from sph_seepage_flows_gb300 import build
    build.build_library()
    root = tmp_path_factory.mktemp("assets")
    g = load_golden("shapes.npz")
    sh = g["shape"]
    (root / "bgeo" / "shapes").mkdir(parents=True)
    (root / "bgeo" / "shapes" / "ball.bgeo").write_bytes(
        bgeo.write_bytes(sh[:, :3], np.zeros((len(sh), 3)), sh[:, 3], np.ones(len(sh))))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    pkg = os.path.join(ROOT, "sph_seepage_flows_gb300")
    out = str(root / "shape_import")
    subprocess.run(["g++", "-std=c++17", "-O2", f'-DDB_PBR_PATH="{root}/"', "-I", os.path.join(ROOT, "include"),
                    "-I", f"{cuda}/include", os.path.join(ROOT, "tests", "cpp", "shape_import.cpp"), "-o", out,
                    "-L", pkg, "-l:libsf_gb300.so", f"-Wl,-rpath,{pkg}", "-L", f"{cuda}/lib64", "-lcudart"],
                   check=True)
    return out


@pytest.mark.parametrize("tag,offset,times", [("plain", 0, 1), ("offset", 1, 1), ("offset_twice", 1, 2)])
def test_shape_volume_import_matches_reference(shape_exe, tag, offset, times):
    """ReadBgeoFileForGPU + BuildSeepageflowShapeMultiVolume equal the
    reference's builder (run on the same points) bit for bit, including the
    offset that moves every particle gathered so far."""
    g = load_golden("shapes.npz")
    r = subprocess.run([shape_exe, "volume", "shapes", "ball", str(offset), "0.02", str(times)],
                       capture_output=True, check=True)
    raw = np.frombuffer(r.stdout, dtype=np.float32)
    assert raw[0] == g[f"{tag}_sand_min_radius"]
    rows = raw[1:].reshape(-1, 14)
    for name, cols in (("pos", slice(0, 3)), ("col", slice(3, 6)), ("cda0asat", slice(6, 9)),
                       ("radius", 9), ("mass", 10), ("amcamcp", slice(11, 13)), ("label", 13)):
        ref = g[f"{tag}_{name}"]
        assert np.array_equal(rows[:, cols], ref.astype(np.float32)), name


def test_boundary_shape_import_matches_reference(shape_exe):
    g = load_golden("shapes.npz")
    r = subprocess.run([shape_exe, "boundary", "shapes", "ball"], capture_output=True, check=True)
    rows = np.frombuffer(r.stdout, dtype=np.float32).reshape(-1, 4)
    assert np.array_equal(rows[:, :3], g["bshape_pos"]) and np.array_equal(rows[:, 3], g["bshape_label"])

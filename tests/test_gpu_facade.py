"""The C++ drop-in facade (include/sf_kiri_facade.hpp): a program written like
the reference app (tests/cpp/facade_main.cpp) compiles against the facade and
libsf_gb300.so, runs one adaptive frame, and ends in the same state as the
Python binding of the C ABI run from the same initial state."""

import subprocess

import numpy as np
import pytest

from helpers import build_facade_program, facade_scene

pytestmark = pytest.mark.gpu


def test_facade_program_matches_c_abi(cuda_lib, tmp_path):
    from sph_seepage_flows_gb300.capi import Simulation
    exe = build_facade_program(tmp_path, "facade_main")
    dump = str(tmp_path / "dump.bin")
    export = tmp_path / "bgeo" / "out"   # the reader's DB_PBR_PATH "bgeo/out"
    out = subprocess.run([exe, dump, "1", str(export)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "facade ok" in out.stdout
    raw = np.fromfile(dump, dtype=np.float32)
    n = raw.size // 6
    init, final = raw[:3 * n].reshape(n, 3), raw[3 * n:].reshape(n, 3)
    sc = facade_scene(init)
    sim = Simulation(sc, capacity=sc.n + 64)
    calls = sim.frame_adaptive(1.0 / 30.0)
    assert f"calls={calls}" in out.stdout
    np.testing.assert_array_equal(sim.field("pos", order="id"), final)
    # ExportBgeoFileCUDA of the final frame: the oracle's bytes for the same
    # arrays in the current (sorted) order, read back by ReadBgeoFileForGPU
    from oracle import bgeo
    data = (export / "0001.bgeo").read_bytes()
    assert data == bgeo.write_bytes(sim.field("pos"), sim.field("col"), sim.field("radius"), sim.field("label"))
    assert f"bgeo read back: {sc.n} points" in out.stdout
    # the searchers' GetCellStartPtr tables equal the C ABI's
    nc = sim.cell_table(0).size
    assert f"cell table 0: entries={nc} last={sc.n} monotone=1" in out.stdout
    assert f"cell table 1: entries={nc} last={sc.nb} monotone=1" in out.stdout

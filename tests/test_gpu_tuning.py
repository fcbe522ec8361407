"""Launch tuning (sf_set_tuning, sf_autotune) changes speed, never results:
every pass computes each slot's outputs independently of the block shape,
so substeps run with any block size are bit-identical. The list capacity
probe sizes the neighbour lists so dense scenes do not overflow them. The
lane count (sf_set_lanes: threads per particle) leaves the lists and every
field up to the momentum passes bit-identical; the momentum sums regroup.
The density pass's shared-memory staging (sf_set_density_staging) changes
where candidates are read from, not which or in what order: lists and
substeps are bit-identical with and without it."""

import numpy as np
import pytest

from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import reference_dt

pytestmark = pytest.mark.gpu

FIELDS = ["pos", "vel", "acc", "density", "pressure", "voidage", "saturation", "avg_flow", "avg_drag",
          "adhesion", "avg_adhesion", "col"]


def run(sc, tune):
    from sph_seepage_flows_gb300.capi import Simulation
    sim = Simulation(sc)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    info = tune(sim, dt)
    sim.substeps_fixed(dt, 4)
    out = {f: sim.field(f, order="id") for f in FIELDS}
    sim.close()
    return out, info


@pytest.mark.parametrize("name", ["tiny", "plain_small"])
def test_block_size_does_not_change_results(cuda_lib, name):
    sc = getattr(scenes, name)()
    ref, _ = run(sc, lambda s, dt: None)
    for bs in (32, 64, 128):
        out, _ = run(sc, lambda s, dt: s.set_tuning(bs))
        for f in FIELDS:
            assert np.array_equal(out[f], ref[f]), (bs, f)
    out, info = run(sc, lambda s, dt: s.autotune(dt))
    assert set(info["block_sizes"].values()) <= {64, 128, 256}
    assert info["density_staged"] in (0, 1)
    assert info["lanes"] in (1, 2, 4, 8) and info["sort_items"] in (1, 2, 4, 8)
    assert 8 <= info["sort_digit_bits"] <= 11
    # the tuner's block sizes and sort tiles change nothing; its lane count
    # regroups the momentum sums, so compare with a run at that lane count
    same_lanes, _ = run(sc, lambda s, dt: s.set_lanes(info["lanes"]))
    for f in FIELDS:
        assert np.array_equal(out[f], same_lanes[f]), ("autotune", f)


def test_list_capacity_covers_dense_scene(cuda_lib):
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scenes.adjoint_column()   # interpenetrating sand / water base: up to ~70 neighbours
    sim = Simulation(sc)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    info = sim.autotune(dt)
    sim.stage("sort")
    sim.stage("density")
    nb = sim.field("neighbors")
    assert info["list_capacity"] % 32 == 0 and info["list_capacity"] >= nb.max() > 64


def test_set_tuning_rejects_bad_sizes(cuda_lib):
    from sph_seepage_flows_gb300.capi import SfError, Simulation
    sim = Simulation(scenes.tiny())
    for bad in (100, 512, -1):
        with pytest.raises(SfError):
            sim.set_tuning(bad)
    with pytest.raises(SfError):
        sim.set_tuning(64, 2)


@pytest.mark.parametrize("name", ["tiny", "plain_small"])
def test_lanes_track_one_lane(cuda_lib, name):
    from sph_seepage_flows_gb300.capi import Simulation
    sc = getattr(scenes, name)()
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    exact = ["density", "pressure", "voidage", "saturation", "avg_flow", "adhesion", "avg_adhesion", "col",
             "max_saturation", "neighbors", "id"]

    def run(lanes):
        sim = Simulation(sc)
        sim.set_lanes(lanes)
        sim.substeps_fixed(dt, 3)  # three full substeps (the momentum passes regroup FP32 sums)
        for st in ("sort", "density", "avgflow", "voidage_adhesion"):
            sim.stage(st, dt)
        out = {f: sim.field(f) for f in exact}
        out["cells"] = sim.cell_table(0)
        sim.stage("sand_momentum", dt)
        sim.stage("water_momentum", dt)
        out["acc"] = sim.field("acc")
        out["pos"] = sim.field("pos")
        sim.close()
        return out

    ref = run(1)
    for lanes in (2, 4, 8, 0):
        out = run(lanes)
        # the states after three substeps differ by momentum rounding only
        # (bit-exactness on identical inputs: the next test)
        assert np.abs(out["pos"] - ref["pos"]).max() < 1e-5, lanes
        scale = np.abs(ref["acc"]).max()
        assert np.abs(out["acc"] - ref["acc"]).max() <= 1e-4 * scale, lanes


def test_lanes_exact_on_identical_inputs(cuda_lib):
    """From one state, the passes up to voidage/adhesion give the same bits for
    every lane count."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scenes.plain_small()
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    fields = ["density", "pressure", "voidage", "saturation", "avg_flow", "adhesion", "avg_adhesion", "col",
              "max_saturation", "neighbors"]
    outs = {}
    for lanes in (1, 2, 4, 8):
        sim = Simulation(sc)
        sim.set_lanes(lanes)
        for st in ("sort", "density", "avgflow", "voidage_adhesion"):
            sim.stage(st, dt)
        outs[lanes] = {f: sim.field(f) for f in fields}
        outs[lanes]["cells"] = sim.cell_table(0)
        sim.close()
    for lanes in (2, 4, 8):
        for f in outs[1]:
            assert np.array_equal(outs[lanes][f], outs[1][f]), (lanes, f)


def test_set_lanes_rejects_bad_counts(cuda_lib):
    from sph_seepage_flows_gb300.capi import SfError, Simulation
    sim = Simulation(scenes.tiny())
    for bad in (3, 16, -1):
        with pytest.raises(SfError):
            sim.set_lanes(bad)


def one_lane(staged, bs):
    def tune(sim, dt):
        sim.set_lanes(1)
        sim.set_tuning(bs)
        sim.set_density_staging(staged)
        assert sim.density_staging() == int(staged)
    return tune


@pytest.mark.parametrize("name", ["tiny", "plain_small"])
def test_density_staging_does_not_change_results(cuda_lib, name):
    """Four substeps with the density candidates staged in shared memory, at
    every block size, equal the unstaged run bit for bit (one thread per
    particle, the path large scenes take)."""
    sc = getattr(scenes, name)()
    ref, _ = run(sc, one_lane(False, 128))
    for bs in (32, 64, 128, 256):
        out, _ = run(sc, one_lane(True, bs))
        for f in FIELDS:
            assert np.array_equal(out[f], ref[f]), (bs, f)


def test_density_staging_identical_lists_at_full_size(cuda_lib):
    """The 1M embankment, where nearly every block stages its candidates:
    neighbour counts, density and pressure of the density stage are the same
    bits with and without staging, at 128 and 256 threads per block (at 256
    the denser blocks exceed the shared capacity and walk global memory)."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scenes.plain_large()
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    outs = {}
    for staged, bs in ((False, 128), (True, 128), (True, 256)):
        sim = Simulation(sc)
        one_lane(staged, bs)(sim, dt)
        sim.stage("sort", dt)
        sim.stage("density", dt)
        outs[(staged, bs)] = {f: sim.field(f) for f in ("neighbors", "density", "pressure", "id")}
        assert sim.check_error() == 0
        sim.close()
    ref = outs[(False, 128)]
    for key in ((True, 128), (True, 256)):
        for f in ref:
            assert np.array_equal(outs[key][f], ref[f]), (key, f)

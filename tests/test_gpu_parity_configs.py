"""Parity at the benchmark configurations themselves, through the C ABI.

* plain_large: the 1,003,499-particle embankment the throughput figures are
  quoted on (500k DEM sand r = 0.005, 500k WCSPH water at pitch 0.01, box
  4.0 x 0.6 x 1.0, h = 0.02, grid 200 x 30 x 50), at the reference dt held
  fixed (2.415e-4 s);
* plain_small: 8,000 sand + 32,000 water in the 1 m box, adaptive substeps;
* a seeded subset of the 64-scene batched ensemble spanning its size range.

Checker: the FP32 CPU oracle (the reference arithmetic) on the same inputs.
Integer results (ids, labels, both cell tables) must be bit-exact, the
fields free of powf and reordered sums bit-for-bit, the rest within the
norm-relative bar of 1e-5 (forces against the oracle's per-particle sum of
term magnitudes). At full size the size-independent properties are checked
as well: the sort is a permutation, the cell tables are monotone with
cellStart[G] = N, the device error word stays clear and no mass is lost.
"""

import numpy as np
import pytest

from helpers import compare_stages, rel_err
from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import reference_dt

pytestmark = pytest.mark.gpu

TOL = 1e-5
T_FRAME = 1.0 / 30.0


@pytest.fixture(scope="module")
def large():
    return scenes.plain_large()


def ref_dt(sc):
    return reference_dt(sc.params, sc.bparams, sc.sparams)[1]


def check_tables(sim, sc, n):
    """Cell tables: start at 0, monotone, end at the live count (particles)
    or the boundary count; the grid has the scene's G cells."""
    g = [int(v) for v in sc.bparams.grid_size]
    G = g[0] * g[1] * g[2]
    for which, total in ((0, n), (1, sc.nb)):
        cs = sim.cell_table(which)
        assert cs.size == G + 1
        assert cs[0] == 0 and cs[-1] == total, (which, cs[0], cs[-1], total)
        assert np.all(np.diff(cs) >= 0), which


def test_plain_large_sort_and_cell_tables_bit_exact(cuda_lib, oracle_mod, large):
    from sph_seepage_flows_gb300.capi import Simulation
    sc = large
    sim = Simulation(sc)
    o32 = oracle_mod.Oracle(sc, 32)
    sim.stage("sort")
    o32.stage("sort")
    ids = sim.field("id")
    assert np.array_equal(np.sort(ids), np.arange(sc.n)), "the sort is not a permutation"
    assert np.array_equal(ids, o32.field("id").astype(np.int32))
    assert np.array_equal(sim.field("label"), o32.field("label").astype(np.int32))
    assert np.array_equal(sim.cell_table(0), o32.cell_table(0))
    assert np.array_equal(sim.cell_table(1), o32.cell_table(1))
    check_tables(sim, sc, sc.n)
    assert sim.check_error() == 0


@pytest.mark.parametrize("lanes", [0])
def test_plain_large_stages_against_fp32_oracle(cuda_lib, oracle_mod, large, lanes):
    """Every stage of two substeps at the reference dt on identical inputs:
    the exact fields bit-for-bit, pressure / adhesion / drag / accelerations
    within 1e-5 (the automatic lane count is 1 at this size)."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = large
    sim = Simulation(sc)
    sim.set_lanes(lanes)
    o32 = oracle_mod.Oracle(sc, 32)
    report = {}
    compare_stages(sim, o32, ref_dt(sc), False, TOL, reps=2, report=report)
    worst = {k: v for k, v in report.items() if v[0] < 1.0}
    print({f"{k[1]}:{k[2]}": (round(f, 5), f"{e:.2e}") for k, (f, e) in worst.items()})
    assert sim.check_error() == 0


def test_plain_large_ten_substeps_track_oracle(cuda_lib, oracle_mod, large):
    """Ten graph-replayed substeps at the reference dt against ten oracle
    substeps from the same initial state: positions by particle id within
    1e-5 m (0.2% of the sand radius), density within 1e-4, and the
    full-size properties (permutation, tables, error word, mass)."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = large
    dt = ref_dt(sc)
    sim = Simulation(sc)
    o32 = oracle_mod.Oracle(sc, 32)
    sim.substeps_fixed(dt, 10)
    o32.substeps(dt, False, 10)
    assert sim.check_error() == 0
    ids = sim.field("id")
    assert np.array_equal(np.sort(ids), np.arange(sc.n))
    check_tables(sim, sc, sc.n)
    mass = sim.field("mass", order="id")
    assert np.array_equal(mass, sc.mass.astype(np.float32)), "mass changed"
    order = np.argsort(o32.field("id"))
    pos = sim.field("pos", order="id").astype(np.float64)
    ref = o32.field("pos")[order]
    d = np.abs(pos - ref).max(1)
    print(f"10 substeps: max |dx| {d.max():.3e} m, 99.9% {np.quantile(d, 0.999):.3e} m")
    assert d.max() < 1e-5
    dens = sim.field("density", order="id")
    assert rel_err(dens, o32.field("density")[order]) < 1e-4


@pytest.mark.parametrize("lanes", [0, 1])
def test_plain_small_stages_against_fp32_oracle(cuda_lib, oracle_mod, lanes):
    """The 40k plain-small scene, two adaptive substeps stage by stage, with
    the automatic lane count and with one thread per particle."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scenes.plain_small()
    sim = Simulation(sc)
    sim.set_lanes(lanes)
    o32 = oracle_mod.Oracle(sc, 32)
    compare_stages(sim, o32, T_FRAME, True, TOL, reps=2)
    check_tables(sim, sc, sc.n)
    assert sim.check_error() == 0


def batched_subset(k=8):
    """k members of the 64-scene ensemble, evenly spread over its sorted sizes."""
    ens = scenes.batched()
    order = np.argsort([s.n for s in ens])
    pick = order[np.linspace(0, len(ens) - 1, k).round().astype(int)]
    return [ens[i] for i in pick]


@pytest.mark.parametrize("lanes", [1, 2, 8])
def test_batched_members_equal_single_scene_handles(cuda_lib, lanes):
    """Eight members of the batched ensemble (2k-60k particles, per-scene
    friction, capillary and permeability) advanced in one handle equal the
    same scenes advanced by their own handles, bit for bit, both with
    graph-replayed fixed-dt blocks and with adaptive substeps, when both run
    the neighbour passes with the same number of threads per particle (the
    momentum sums' FP32 order depends on it)."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = batched_subset()
    sizes = [s.n for s in sc]
    assert min(sizes) < 4000 and max(sizes) > 40000, sizes
    dt = ref_dt(sc[0])
    batch = Simulation(sc)
    singles = [Simulation(s) for s in sc]
    for h in [batch] + singles:
        h.set_lanes(lanes)
    batch.substeps_fixed(dt, 20)
    for s in singles:
        s.substeps_fixed(dt, 20)
    for _ in range(2):
        batch.step(T_FRAME)
        for s in singles:
            s.step(T_FRAME)
    assert batch.check_error() == 0
    for k, s in enumerate(singles):
        assert batch.num_substeps(k) == s.num_substeps(), k
        for name in ("pos", "vel", "acc", "density", "saturation", "id"):
            assert np.array_equal(batch.field(name, scene=k), s.field(name)), (k, sizes[k], name)
        assert np.array_equal(batch.cell_table(0, scene=k), s.cell_table(0)), k


def test_batched_members_track_single_scene_handles_with_automatic_lanes(cuda_lib):
    """With the automatic lane counts (fewer threads per particle in the
    batched handle than in a small scene's own handle) the members follow
    their single-scene runs within FP32 rounding: positions by id within
    1e-6 m after 20 substeps."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = batched_subset()
    dt = ref_dt(sc[0])
    batch = Simulation(sc)
    singles = [Simulation(s) for s in sc]
    batch.substeps_fixed(dt, 20)
    worst = 0.0
    for k, s in enumerate(singles):
        s.substeps_fixed(dt, 20)
        d = np.abs(batch.field("pos", order="id", scene=k) - s.field("pos", order="id")).max()
        worst = max(worst, float(d))
    print(f"lanes batch {batch.tuning()['lanes']} singles {[s.tuning()['lanes'] for s in singles]}: "
          f"max |dx| {worst:.3e} m")
    assert worst < 1e-6


def test_batched_member_stages_against_fp32_oracle(cuda_lib, oracle_mod):
    """The largest member of the subset, stage by stage against the oracle
    (the chain batch = single = oracle at a size the small fixtures miss)."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = max(batched_subset(), key=lambda s: s.n)
    sim = Simulation(sc)
    o32 = oracle_mod.Oracle(sc, 32)
    compare_stages(sim, o32, ref_dt(sc), False, TOL, reps=1)

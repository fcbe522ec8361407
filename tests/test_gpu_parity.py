"""Parity of the CUDA substep (through the C ABI) with the reference.

Checkers: the golden fixtures written by tests/golden/make_golden.py from the
reference's own kernels, and the CPU oracle (FP32 = the reference arithmetic,
FP64 = the error yardstick) on the same inputs.

Tolerances. Integer and index results (sort order, ids, labels, cell tables)
must be bit-exact. Floating-point results are compared with the norm-relative
error |gpu - ref| / scale, scale = the per-particle magnitude of the quantity
(for acceleration: the sum of the magnitudes of all terms added to it, from
the FP64 oracle; for pressure: stiff * (rho/rho0)^7), with a floor of 1e-3 of
the field's largest scale. The bar is 1e-5: forces within 1e-5 relative of
the reference's FP32 path. Fields
computed without transcendental functions must match the FP32 oracle
bit-for-bit when the inputs are identical.
"""

import numpy as np
import pytest

from helpers import compare_stages, exact_fraction, load_golden, rel_err, scene_from_golden
from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import STAGES

pytestmark = pytest.mark.gpu

TOL = 1e-5
T_FRAME = 1.0 / 30.0
FLOAT_FIELDS = ["pos", "vel", "acc", "col", "density", "pressure", "voidage", "saturation", "max_saturation",
                "avg_flow", "avg_drag", "adhesion", "avg_adhesion"]


def gpu_sim(scene, **kw):
    from sph_seepage_flows_gb300.capi import Simulation
    return Simulation(scene, **kw)


def yardsticks(oracle_mod, scene, stage_fn):
    """FP64 oracle scales for acc and pressure after running stage_fn(o64)."""
    o64 = oracle_mod.Oracle(scene, 64)
    stage_fn(o64)
    return o64


def field_scale(name, o64, n):
    if o64 is None:
        return None
    if name == "acc":
        return o64.field("acc_scale")
    if name == "pressure":
        return o64.field("pressure_scale")
    return None


def test_sort_and_cell_table_bit_exact(cuda_lib):
    g = load_golden("tiny_multi_wcsph.npz")
    sim = gpu_sim(scene_from_golden(g))
    sim.stage("sort")
    assert np.array_equal(sim.cell_table(0), g["s1_cell_start"].astype(np.int64))
    assert np.array_equal(sim.field("id"), g["s1_id"])
    assert np.array_equal(sim.field("label"), g["s1_label"])
    assert np.array_equal(sim.cell_table(1), g["bcell_start"].astype(np.int64))
    np.testing.assert_array_equal(sim.field("bpos"), g["bpos_sorted"])


def test_boundary_volume_matches_reference(cuda_lib):
    g = load_golden("tiny_multi_wcsph.npz")
    sim = gpu_sim(scene_from_golden(g))
    bv = sim.field("bvolume")
    assert exact_fraction(bv, g["bvolume"]) == 1.0


@pytest.mark.parametrize("fixture", ["tiny_multi_wcsph.npz", "tiny_sf_sph.npz"])
def test_one_substep_matches_reference_kernels(cuda_lib, oracle_mod, fixture):
    g = load_golden(fixture)
    scene = scene_from_golden(g)
    sim = gpu_sim(scene)
    nsub = sim.step(T_FRAME)
    assert nsub == int(g["s1_n_sub"])
    o64 = yardsticks(oracle_mod, scene, lambda o: o.substeps(T_FRAME, True, 1))
    assert np.array_equal(sim.field("id"), g["s1_id"])
    assert np.array_equal(sim.cell_table(0), g["s1_cell_start"].astype(np.int64))
    report = {}
    for name in FLOAT_FIELDS:
        got, ref = sim.field(name), g["s1_" + name]
        report[name] = (exact_fraction(got, ref), rel_err(got, ref, field_scale(name, o64, scene.n)))
    print({k: (round(a, 4), f"{b:.2e}") for k, (a, b) in report.items()})
    for name, (_, err) in report.items():
        assert err <= TOL, (name, err)


def dense_cluster_scene():
    """Sand compressed to 0.3x its lattice pitch: ~1000 neighbours per
    particle, far above the neighbour-list capacity (stencil fallback)."""
    sc = scenes.tiny(seed=12, sand=(8, 8, 8), water=(4, 6, 6))
    sand = sc.label == 1
    c = sc.pos[sand].mean(0)
    sc.pos = sc.pos.copy()
    sc.pos[sand] = (c + 0.3 * (sc.pos[sand] - c)).astype(np.float32)
    return sc


@pytest.mark.parametrize("lanes", [0, 1])
@pytest.mark.parametrize("which", ["tiny", "dense", "plate"])
def test_stages_bit_exact_against_fp32_oracle(cuda_lib, oracle_mod, which, lanes):
    """Each stage on identical inputs: the GPU output equals the FP32 oracle's
    bit-for-bit for every field free of powf and of reordered sums, within TOL
    otherwise. "dense" exercises the neighbour-list overflow fallback, "plate"
    the shape boundary particles (label 1: sand DEM, water push-out). lanes 0
    is the automatic choice for these small scenes (8 threads per particle);
    lanes 1 is the one-thread-per-particle path that large scenes take."""
    sc = {"tiny": lambda: scenes.tiny(seed=11), "dense": dense_cluster_scene,
          "plate": scenes.tiny_with_plate}[which]()
    sim = gpu_sim(sc)
    sim.set_lanes(lanes)
    o32 = oracle_mod.Oracle(sc, 32)
    compare_stages(sim, o32, T_FRAME, True, TOL, reps=2 if which == "tiny" else 1)


def test_fields_set_between_stages_reach_the_momentum_passes(cuda_lib, oracle_mod):
    """sf_set_field between the voidage/adhesion pass and the momentum passes:
    the values the passes derived from the changed fields (the water (D, P)
    pairs, the gather records, the adhesion Bezier factor) are recomputed, so
    the momentum passes see the new fields as the reference's kernels would."""
    sc = scenes.tiny(seed=13)
    sim = gpu_sim(sc)
    o32 = oracle_mod.Oracle(sc, 32)
    for st in ("sort", "density", "avgflow", "voidage_adhesion"):
        sim.stage(st, T_FRAME, adaptive=True)
        o32.stage(st, T_FRAME, adaptive=True)
    for name in ("pos", "vel", "density", "pressure", "voidage", "saturation", "avg_flow", "adhesion",
                 "avg_adhesion", "col", "max_saturation"):
        o32.set_field(name, sim.field(name))
    rng = np.random.default_rng(5)
    n = sc.n
    sand = sim.field("label") == 1
    vel = (sim.field("vel") + rng.normal(0, 0.05, (n, 3))).astype(np.float32)
    sat = np.where(sand, rng.random(n), sim.field("saturation")).astype(np.float32)
    prs = (sim.field("pressure") * rng.uniform(0.9, 1.1, n)).astype(np.float32)
    void = np.where(sand, rng.uniform(0.35, 0.65, n), rng.uniform(0.5, 1.0, n)).astype(np.float32)
    dens = (sim.field("density") * np.where(sand, 1.0, rng.uniform(0.98, 1.02, n))).astype(np.float32)
    for name, v in (("vel", vel), ("saturation", sat), ("pressure", prs), ("voidage", void), ("density", dens)):
        sim.set_field(name, v)
        o32.set_field(name, v)
    for st, lab in (("sand_momentum", 1), ("water_momentum", 0)):
        sim.stage(st, T_FRAME, adaptive=True)
        o32.stage(st, T_FRAME, adaptive=True)
        keep = sim.field("label") == lab
        err = rel_err(sim.field("acc")[keep], o32.field("acc")[keep], o32.field("acc_scale")[keep])
        assert err <= TOL, (st, err)


def test_ten_substeps_track_reference(cuda_lib):
    g = load_golden("tiny_multi_wcsph.npz")
    sim = gpu_sim(scene_from_golden(g))
    for _ in range(10):
        sim.step(T_FRAME)
    ids = sim.field("id")
    assert np.array_equal(np.sort(ids), np.sort(g["s10_id"]))
    order = np.argsort(ids)
    ref_order = np.argsort(g["s10_id"])
    pos, ref = sim.field("pos")[order], g["s10_pos"][ref_order]
    # positions agree to well below a particle radius (0.01) after 10 substeps
    assert np.abs(pos - ref).max() < 1e-6
    dens = sim.field("density")[order]
    assert rel_err(dens, g["s10_density"][ref_order]) < 1e-4


def test_shape_plate_substep_tracks_reference(cuda_lib):
    """One adaptive substep on the shape-boundary plate scene against the
    reference kernels' fixture (tiny_plate.npz)."""
    g = load_golden("tiny_plate.npz")
    sim = gpu_sim(scene_from_golden(g))
    sim.step(T_FRAME)
    assert sim.num_substeps() == int(g["s1_n_sub"])
    order, ref_order = np.argsort(sim.field("id")), np.argsort(g["s1_id"])
    assert np.abs(sim.field("pos")[order] - g["s1_pos"][ref_order]).max() < 1e-6
    assert np.array_equal(sim.cell_table(0), g["s1_cell_start"].astype(np.int64))


def test_fixed_dt_graph_equals_eager(cuda_lib):
    sc = scenes.tiny(seed=3)
    a, b = gpu_sim(sc), gpu_sim(sc)
    dt = 4.8e-4
    a.substeps_fixed(dt, 6)
    for _ in range(6):
        for st in STAGES:
            b.stage(st, dt, adaptive=False)
    for name in ("pos", "vel", "acc", "density", "id"):
        assert np.array_equal(a.field(name), b.field(name)), name


def test_deterministic(cuda_lib):
    sc = scenes.tiny(seed=4)
    a, b = gpu_sim(sc), gpu_sim(sc)
    for s in (a, b):
        for _ in range(5):
            s.step(T_FRAME)
    for name in ("pos", "vel", "acc", "col", "id"):
        assert np.array_equal(a.field(name), b.field(name)), name


def test_batched_equals_single(cuda_lib):
    sc = [scenes.tiny(seed=21), scenes.tiny(seed=22, sand=(6, 6, 6), water=(5, 9, 7)), scenes.tiny(seed=23)]
    sc[2].params.dem_tan_friction_angle = 0.7
    batch = gpu_sim(sc)
    singles = [gpu_sim(s) for s in sc]
    for _ in range(3):
        batch.step(T_FRAME)
        for s in singles:
            s.step(T_FRAME)
    for k, s in enumerate(singles):
        for name in ("pos", "vel", "acc", "density", "id"):
            assert np.array_equal(batch.field(name, scene=k), s.field(name)), (k, name)


def test_adaptive_frame_matches_oracle(cuda_lib, oracle_mod):
    sc = scenes.tiny(seed=5)
    sim = gpu_sim(sc)
    o = oracle_mod.Oracle(sc, 32)
    calls = sim.frame_adaptive(0.005)
    assert calls == o.frame_adaptive(0.005)
    order, oorder = np.argsort(sim.field("id")), np.argsort(o.field("id"))
    assert np.abs(sim.field("pos")[order] - o.field("pos")[oorder]).max() < 1e-6


def test_add_sph_particles_and_capacity(cuda_lib):
    sc = scenes.tiny(seed=6)
    sim = gpu_sim(sc, capacity=sc.n + 100)
    pts = np.array([[0.1, 0.3, 0.2], [0.12, 0.3, 0.2]], np.float32)
    sim.add_sph_particles(pts, [0.5, 0.8, 1.0], [0.0, -1.0, 0.0], sc.params.sph_mass, sc.params.sph_particle_radius)
    assert sim.size() == sc.n + 2
    sim.step(T_FRAME)
    ids = sim.field("id", order="id")
    assert np.array_equal(ids, np.arange(sc.n + 2))
    from sph_seepage_flows_gb300.capi import SfError
    with pytest.raises(SfError):
        sim.add_sph_particles(np.zeros((98, 3), np.float32), [0, 0, 1], [0, 0, 0], 1.0, 0.01)
    assert sim.size() == sc.n + 2


def test_device_error_word_reports_nonfinite(cuda_lib):
    sc = scenes.tiny(seed=8)
    sim = gpu_sim(sc)
    pos = sim.field("pos")
    pos[0, 1] = np.nan
    sim.set_field("pos", pos)
    sim.step(T_FRAME)
    flags = sim.check_error()
    assert flags & 1


def test_pinned_host_fields_match_staged(cuda_lib):
    """Fields read into / written from page-locked host memory (read and
    written by the kernels directly) equal the staged copies, bit for bit."""
    torch = pytest.importorskip("torch")
    sc = scenes.tiny()
    sim = gpu_sim(sc)
    sim.substeps_fixed(2.0e-4, 3)
    for name in ("pos", "vel", "density", "label"):
        ref = sim.field(name)
        pinned = torch.empty(ref.shape, dtype=getattr(torch, str(ref.dtype)), pin_memory=True).numpy()
        sim.field(name, out=pinned)
        assert np.array_equal(pinned, ref), name
    pinned = torch.empty((sc.n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pinned[:] = sim.field("vel") * np.float32(0.5)
    sim.set_field("vel", pinned)
    assert np.array_equal(sim.field("vel"), pinned)


def test_multi_field_calls_equal_single_field_calls(cuda_lib):
    """sf_set_fields / sf_get_fields (one wait for several fields), with pinned
    and pageable host buffers, in both orders, equal the one-field calls."""
    torch = pytest.importorskip("torch")
    sc = scenes.tiny(seed=5)
    a, b = gpu_sim(sc), gpu_sim(sc)
    for s in (a, b):
        s.substeps_fixed(2.0e-4, 3)
    rng = np.random.default_rng(2)
    for order in ("sorted", "id"):
        new = {"pos": (a.field("pos", order) + rng.normal(0, 1e-4, (sc.n, 3))).astype(np.float32),
               "vel": rng.normal(0, 0.1, (sc.n, 3)).astype(np.float32),
               "saturation": rng.random(sc.n).astype(np.float32)}
        for k, v in new.items():
            a.set_field(k, v, order)
        pinned = {}
        for k, v in new.items():
            pinned[k] = torch.empty(v.shape, dtype=torch.float32, pin_memory=True).numpy()
            pinned[k][:] = v
        b.set_fields(pinned if order == "sorted" else new, order)
        outs = {k: torch.empty(v.shape, dtype=torch.float32, pin_memory=True).numpy() for k, v in new.items()}
        b.get_fields(outs, order)
        for k in new:
            assert np.array_equal(outs[k], a.field(k, order)), (order, k)
        a.substeps_fixed(2.0e-4, 2)
        b.substeps_fixed(2.0e-4, 2)
        assert np.array_equal(a.field("pos", "id"), b.field("pos", "id")), order

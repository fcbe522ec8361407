"""The oracle against the golden fixtures of the reference kernels
(tests/golden/, written by tests/golden/make_golden.py). CPU only."""

import numpy as np
import pytest

from helpers import load_golden, rel_err, scene_from_golden
from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import FIELDS

T = 1.0 / 30.0
NAMES = [k for k in FIELDS if k not in ("key", "neighbors")]


@pytest.mark.parametrize("fixture", ["tiny_multi_wcsph.npz", "tiny_sf_sph.npz", "tiny_plate.npz"])
def test_fp32_oracle_bit_exact_after_one_substep(oracle_mod, fixture):
    g = load_golden(fixture)
    o = oracle_mod.Oracle(scene_from_golden(g), 32)
    o.substeps(T, True, 1)
    assert o.num_substeps == int(g["s1_n_sub"])
    assert np.array_equal(o.cell_table(0), g["s1_cell_start"].astype(np.int64))
    for name in NAMES:
        got = o.field(name)
        ref = g["s1_" + name].astype(np.float64)
        assert np.array_equal(got, ref), name


def test_fp32_oracle_bit_exact_after_ten_substeps(oracle_mod):
    g = load_golden("tiny_multi_wcsph.npz")
    o = oracle_mod.Oracle(scene_from_golden(g), 32)
    o.substeps(T, True, 10)
    for name in ("id", "label", "pos", "vel", "acc", "density", "pressure", "voidage", "saturation",
                 "max_saturation", "col"):
        assert np.array_equal(o.field(name), g["s10_" + name].astype(np.float64)), name


def test_boundary_volume_and_cell_table(oracle_mod):
    g = load_golden("tiny_multi_wcsph.npz")
    o = oracle_mod.Oracle(scene_from_golden(g), 32)
    assert np.array_equal(o.cell_table(1), g["bcell_start"].astype(np.int64))
    assert np.array_equal(o.field("bvolume"), g["bvolume"].astype(np.float64))
    assert np.array_equal(o.field("bpos"), g["bpos_sorted"].astype(np.float64))


def test_fp64_oracle_close_to_fp32_reference(oracle_mod):
    """The FP64 yardstick stays within FP32 rounding of the reference after
    one substep (acceleration measured against the sum of term magnitudes)."""
    g = load_golden("tiny_multi_wcsph.npz")
    o = oracle_mod.Oracle(scene_from_golden(g), 64)
    o.substeps(T, True, 1)
    assert np.array_equal(o.field("id"), g["s1_id"].astype(np.float64))
    assert rel_err(o.field("density"), g["s1_density"]) < 1e-6
    assert rel_err(g["s1_acc"], o.field("acc"), o.field("acc_scale")) < 1e-4
    assert np.abs(o.field("pos") - g["s1_pos"]).max() < 1e-7


def test_fixture_inputs_match_generator():
    g = load_golden("tiny_multi_wcsph.npz")
    sc = scenes.tiny()
    for k in ("pos", "col", "label", "mass", "radius", "cda0asat", "amcamcp", "bpos", "blabel"):
        assert np.array_equal(getattr(sc, k), g["in_" + k]), k
    assert bytes(sc.params) == g["params"].tobytes()
    assert bytes(sc.bparams) == g["bparams"].tobytes()


def test_world_boundary_matches_reference_emitter():
    e = load_golden("emitters.npz")
    pos, lab = scenes.world_boundary((0.0, 0.0, 0.0), (0.4, 0.4, 0.4), 0.01)
    assert np.array_equal(pos, e["world_boundary_small"])
    assert np.array_equal(lab, e["world_boundary_small_label"])
    big, _ = scenes.world_boundary((0.0, 0.0, 0.0), (4.0, 0.6, 1.0), 0.005)
    assert big.shape[0] == int(e["world_boundary_large_count"])
    np.testing.assert_allclose(big.astype(np.float64).sum(0), e["world_boundary_large_sum"], rtol=1e-12)

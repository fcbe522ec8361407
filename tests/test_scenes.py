"""Seeded scene generator: counts, determinism, layout invariants."""

import numpy as np

from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import reference_dt


def test_plain_small_counts_and_box():
    sc = scenes.plain_small()
    assert sc.n_sand == 8000 and sc.n_water == 32000
    assert list(sc.bparams.grid_size) == [25, 25, 25]
    assert (sc.pos >= 0).all() and (sc.pos <= 1).all()
    n_sub, dt = reference_dt(sc.params, sc.bparams, sc.sparams)
    assert n_sub == 69 and abs(dt - 4.831e-4) < 1e-6


def test_plain_large_counts_within_half_percent():
    sc = scenes.plain_large()
    assert abs(sc.n_sand - 500_000) <= 2500 and abs(sc.n_water - 500_000) <= 2500
    assert list(sc.bparams.grid_size) == [200, 30, 50]
    n_sub, dt = reference_dt(sc.params, sc.bparams, sc.sparams)
    assert n_sub == 138 and abs(dt - 2.415e-4) < 1e-6


def test_seeded_generation_is_deterministic():
    a, b = scenes.plain_small(seed=5), scenes.plain_small(seed=5)
    assert np.array_equal(a.pos, b.pos)
    c = scenes.plain_small(seed=6)
    assert not np.array_equal(a.pos, c.pos)


def test_batched_scene_parameters_in_range():
    sc = scenes.batched(n_scenes=8, seed=3)
    for s in sc:
        assert 1000 <= s.n <= 80000
        phi = np.degrees(np.arctan(s.params.dem_tan_friction_angle))
        assert 24.9 <= phi <= 40.1
        assert 0.5 <= s.meta["cap_scale"] <= 2.0 and 0.5 <= s.meta["perm_scale"] <= 2.0

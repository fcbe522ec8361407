"""Pins the oracle to the reference's own kernels run on the CPU (the
reference harness, oracle/_ref/libsfref.so). Runs only where the reference
sources are mounted and the harness is built; the golden fixtures carry the
same pin elsewhere."""

import numpy as np
import pytest

from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import FIELDS, SF_SOLVER_SPH, SF_TYPE_SF

T = 1.0 / 30.0


@pytest.fixture(scope="module")
def harness(oracle_mod):
    if oracle_mod.ref_lib() is None:
        pytest.skip("reference harness not built (reference sources not mounted)")
    return oracle_mod


CASES = [
    ("multi_wcsph", dict(seed=31), None),
    ("sf_wcsph", dict(seed=32), dict(sf_type=SF_TYPE_SF)),
    ("multi_sph", dict(seed=33), dict(solver_type=SF_SOLVER_SPH)),
    ("sf_sph_friction", dict(seed=34, sand=(6, 10, 6), water=(9, 8, 9)),
     dict(sf_type=SF_TYPE_SF, solver_type=SF_SOLVER_SPH, dem_tan_friction_angle=0.9, sf_cd=0.2)),
]


@pytest.mark.parametrize("name,kw,override", CASES, ids=[c[0] for c in CASES])
def test_oracle_bit_exact_with_reference_kernels(harness, name, kw, override):
    sc = scenes.tiny(**kw)
    for k, v in (override or {}).items():
        setattr(sc.params, k, v)
    ref = harness.RefHarness(sc)
    o = harness.Oracle(sc, 32)
    for step in range(4):
        ref.substeps(T, True, 1)
        o.substeps(T, True, 1)
        assert o.num_substeps == ref.num_substeps
        assert np.array_equal(o.cell_table(0), ref.cell_table(0))
        for f in FIELDS:
            if f in ("key", "neighbors"):
                continue
            assert np.array_equal(o.field(f), ref.field(f)), (step, f)


def test_shape_boundary_plate(harness):
    """Shape boundary particles (label 1): sand DEM against them and the
    water push-out of the integrator."""
    sc = scenes.tiny_with_plate()
    assert (sc.blabel == 1).sum() > 1000
    ref = harness.RefHarness(sc)
    o = harness.Oracle(sc, 32)
    for step in range(4):
        ref.substeps(T, True, 1)
        o.substeps(T, True, 1)
        assert o.num_substeps == ref.num_substeps
        for f in FIELDS:
            if f in ("key", "neighbors"):
                continue
            assert np.array_equal(o.field(f), ref.field(f)), (step, f)


def test_moving_water_column_with_velocities(harness):
    sc = scenes.tiny(seed=35)
    rng = np.random.default_rng(0)
    sc.vel = rng.normal(0, 0.3, sc.pos.shape).astype(np.float32)
    ref = harness.RefHarness(sc)
    o = harness.Oracle(sc, 32)
    ref.substeps(T, True, 3)
    o.substeps(T, True, 3)
    for f in ("pos", "vel", "acc", "avg_flow", "avg_drag", "adhesion", "voidage"):
        assert np.array_equal(o.field(f), ref.field(f)), f


def test_reference_emitters(harness):
    lo, hi = (0.0, 0.0, 0.0), (1.0, 0.5, 0.7)
    pos, lab = harness.ref_world_boundary(lo, hi, 0.01)
    mine, ml = scenes.world_boundary(lo, hi, 0.01)
    assert np.array_equal(pos, mine) and np.array_equal(lab, ml)

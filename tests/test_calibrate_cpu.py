"""Host logic of the batched calibration (no GPU): parameter scaling, the
Adam update and the calibration scenes."""

import numpy as np

from sph_seepage_flows_gb300 import calibrate, scenes
from sph_seepage_flows_gb300.params import SF_LABEL_SAND


def test_scene_params_scale_capillary_and_cd():
    sc = scenes.column_scene("c", 500, 400, 3)
    p = calibrate.scene_params(sc, (0.6, 1.5, 0.5))
    assert np.float32(p.dem_tan_friction_angle) == np.float32(0.6)
    assert np.float32(p.sf_c0) == np.float32(sc.params.sf_c0 * 1.5)
    assert np.float32(p.sf_cmc) == np.float32(sc.params.sf_cmc * 1.5)
    assert np.float32(p.sf_cd) == np.float32(sc.params.sf_cd * 0.5)
    assert sc.params.sf_c0 == np.float32(0.7)  # the base scene is untouched


def test_adam_descends_a_quadratic():
    opt = calibrate.Adam((3,), lr=0.1)
    x = np.array([1.0, -2.0, 3.0])
    for _ in range(200):
        x = opt.step(x, 2.0 * x)
    assert np.abs(x).max() < 0.05


def test_calibration_workload_shapes():
    scs, theta0, theta_true, dt = calibrate.workload(n_scenes=4)
    assert len(scs) == 4 and theta0.shape == (4, 3) and theta_true.shape == (4, 3)
    assert np.all(np.abs(theta_true / theta0 - 1) <= 0.1 + 1e-12)
    assert dt > 0
    for sc in scs:
        lo = np.asarray(sc.bparams.lowest_point[:])
        hi = np.asarray(sc.bparams.highest_point[:])
        assert np.all(sc.pos > lo) and np.all(sc.pos < hi)
        assert 0.3 < (sc.label == SF_LABEL_SAND).mean() < 0.7
    geos = {sc.meta["geometry"] for sc in scs}
    assert geos == {"column", "embankment"}


def test_calibration_scene_sizes():
    scs = scenes.calibration_scenes()
    n = np.array([s.n for s in scs])
    assert len(scs) == 32 and n.min() >= 9_000 and n.max() <= 55_000


def test_seed_scales_shrink_only_where_the_gradient_overflowed():
    s = calibrate.next_seed_scales([1.0, 1.0, 2.0 ** -40, 2.0 ** -90], [True, False, False, False])
    assert s[0] == 1.0
    assert s[1] == 2.0 ** -40 and s[2] == 2.0 ** -80
    assert s[3] == calibrate.SEED_FLOOR  # never below the floor
    assert all(np.log2(v).is_integer() for v in s)  # powers of two: no rounding changes

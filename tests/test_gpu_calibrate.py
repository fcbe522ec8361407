"""Batched calibration through the adjoint (calibrate.py) on the GPU: two
small scenes of the calibration geometries (column collapse, embankment
seepage) in one handle recover parameters perturbed by up to 10% from the
loss of their final sand positions."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_calibration_reduces_every_scene_loss(cuda_lib):
    from sph_seepage_flows_gb300 import calibrate, scenes
    from sph_seepage_flows_gb300.params import reference_dt
    scs = [scenes.column_scene("column", 1200, 1000, 1), scenes.embankment_scene("embankment", 1200, 1200, 2)]
    dt = reference_dt(scs[0].params, scs[0].bparams, scs[0].sparams)[1]
    theta0 = np.array([[s.params.dem_tan_friction_angle, 1.0, 1.0] for s in scs])
    theta_true = theta0 * np.array([[1.1, 0.9, 1.1], [0.92, 1.1, 0.9]])
    n_sub = 24
    targets = calibrate.forward_targets(scs, theta_true, dt, n_sub)
    h = calibrate.calibrate(scs, targets, theta0, dt, n_sub, checkpoint_every=8, iterations=8, lr=0.03)
    loss = np.array(h["loss"])
    assert np.all(np.isfinite(loss))
    assert np.all(loss[-1] < loss[0]), loss[:, :]
    assert loss[-1].mean() < 0.7 * loss[0].mean(), loss.mean(1)

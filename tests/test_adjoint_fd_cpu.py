"""The finite-difference references of the adjoint tests are well posed.

The reference model has value discontinuities (liquid-bridge onset and
rupture, voidage onset, the sign switch of the sand damping, the water
velocity clamp), across which a pathwise gradient and a finite difference
disagree. The probe scenes keep every pair away from them over the tested
horizons; here the FP64 oracle confirms that central differences at two
step sizes agree, which is the precondition of the GPU comparisons in
test_gpu_adjoint.py.
"""

import numpy as np
import pytest

from fd_oracle import (CONTACT_CASES, DT, PROBE_CASES, STEPS, contact_scene, directional_state, jvp,
                       param_derivative, probe_direction, probe_scene, probe_target)
from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import SF_LABEL_SAND, SF_LABEL_WATER


def test_probe_scene_margins():
    sc = scenes.adjoint_probe()
    h = sc.params.sph_kernel_radius
    sand = sc.pos[sc.label == SF_LABEL_SAND].astype(np.float64)
    water = sc.pos[sc.label == SF_LABEL_WATER].astype(np.float64)
    d = np.linalg.norm(water[:, None] - sand[None], axis=2)
    assert np.all(np.abs(d - 0.5 * h) >= 5e-4) and np.all(np.abs(d - h) >= 5e-4)
    ds = np.linalg.norm(sand[:, None] - sand[None], axis=2) + np.eye(len(sand))
    gap = ds - 2 * sc.params.dem_particle_radius
    srupt = scenes.capillary_rupture(sc.params.dem_particle_radius)
    near = gap < 2 * srupt
    assert np.all(gap[near] > 0.2 * srupt) and np.all(gap[near] < 0.8 * srupt)  # inside the bridge band
    assert sc.n_sand == 75 and 200 < sc.n_water < 240


@pytest.mark.parametrize("seed,n_sub,damping", PROBE_CASES)
def test_fd_reference_converges(oracle_mod, seed, n_sub, damping):
    sc = probe_scene(seed, damping)
    target = probe_target(sc)
    u = probe_direction(sc, seed)
    for which in ("pos", "vel"):
        a, b = (directional_state(oracle_mod, sc, DT, n_sub, target, which, u, h) for h in STEPS[which])
        assert abs(a - b) <= 1e-5 * abs(b), (which, a, b)
    for which in ("tan", "cap", "perm"):
        a, b = (param_derivative(oracle_mod, sc, DT, n_sub, target, which, h) for h in STEPS[which])
        assert abs(a - b) <= 1e-4 * abs(b), (which, a, b)


@pytest.mark.parametrize("seed,n_sub,damping", PROBE_CASES)
def test_forward_mode_oracle_matches_fd(oracle_mod, seed, n_sub, damping):
    """The FP64 forward-mode oracle (the reference gradient of the GPU
    adjoint tests) agrees with converged central differences."""
    sc = probe_scene(seed, damping)
    target = probe_target(sc)
    u = probe_direction(sc, seed)
    for which in ("pos", "vel"):
        fd = directional_state(oracle_mod, sc, DT, n_sub, target, which, u, STEPS[which][1])
        assert abs(jvp(oracle_mod, sc, DT, n_sub, target, which, u) - fd) <= 1e-6 * abs(fd)
    for which in ("tan", "cap", "perm"):
        fd = param_derivative(oracle_mod, sc, DT, n_sub, target, which, STEPS[which][1])
        # the capillary FD perturbs float32-rounded c0 / cmc (relative rounding ~1e-5 of the step)
        assert abs(jvp(oracle_mod, sc, DT, n_sub, target, which) - fd) <= 5e-5 * abs(fd)


@pytest.mark.parametrize("seed,n_sub,overlap,speed", CONTACT_CASES)
def test_forward_mode_oracle_on_contact_probes(oracle_mod, seed, n_sub, overlap, speed):
    """DEM-contact probes: the forward-mode oracle agrees with central
    differences at the fine step to the ~1e-4 that the friction-cap kinks
    crossed within one step leave in the differences."""
    sc = contact_scene(seed, overlap, speed)
    target = probe_target(sc)
    u = probe_direction(sc, seed)
    for which in ("pos", "vel"):
        fd = directional_state(oracle_mod, sc, DT, n_sub, target, which, u, STEPS[which][1])
        assert abs(jvp(oracle_mod, sc, DT, n_sub, target, which, u) - fd) <= 1e-3 * abs(fd)
    for which in ("tan", "perm"):
        fd = param_derivative(oracle_mod, sc, DT, n_sub, target, which, STEPS[which][1])
        assert abs(jvp(oracle_mod, sc, DT, n_sub, target, which) - fd) <= 5e-4 * abs(fd)

"""FP64 central finite differences of the trajectory loss on the CPU oracle:
the reference values for the GPU adjoint (sf_adjoint_run).

L = mean over sand of |x_T - target|^2 after T substeps at a fixed dt. The
parameter directions follow the adjoint's definitions: tan friction angle,
a capillary scale multiplying c0 / cmc / csat and a permeability scale
multiplying cd (the scene parameter and the per-particle cd of MULTI scenes).
"""

from __future__ import annotations

import copy

import numpy as np

from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import SF_LABEL_SAND

DT = 2e-4
# (seed, substeps, damping) of the probe trajectories; with the reference's
# damping 0.4 the sign switch of the damping is met after ~10 substeps
PROBE_CASES = [(11, 8, 0.4), (12, 8, 0.0), (11, 24, 0.0)]
TARGET_SHIFT = np.array([0.004, -0.002, 0.003])


def probe_scene(seed, damping):
    sc = scenes.adjoint_probe(seed=seed)
    sc.params.dem_damping = damping
    return sc


# (seed, substeps, sand overlap, random sand speed) of the DEM-contact probes:
# every sand lattice pair overlapping (no liquid bridges), sliding contacts,
# no damping. Their loss has friction-cap kinks, so central differences
# converge only at the fine step; the forward-mode oracle is their reference.
CONTACT_CASES = [(21, 8, 4e-4, 0.02), (22, 8, 6e-4, 0.03)]


def contact_scene(seed, overlap, speed):
    sc = scenes.adjoint_probe(seed=seed, sand_overlap=overlap, sand_speed=speed, sand_velocity=(0.0, 0.0, 0.0))
    sc.params.dem_damping = 0.0
    return sc


def probe_target(scene):
    return scene.pos.astype(np.float64) + TARGET_SHIFT


def probe_direction(scene, seed):
    return np.random.default_rng(seed).standard_normal(scene.pos.shape)


def loss(oracle_mod, scene, dt, n_sub, target, pos=None, vel=None) -> float:
    o = oracle_mod.Oracle(scene, precision=64)
    if pos is not None:   # before the first sort the oracle holds the creation (id) order
        o.set_field("pos", pos)
    if vel is not None:
        o.set_field("vel", vel)
    o.substeps(dt, False, n_sub)
    p = o.field("pos")
    ids = o.field("id").astype(np.int64)
    x = np.empty_like(p)
    x[ids] = p
    sand = scene.label == SF_LABEL_SAND
    return float(np.mean(np.sum((x[sand] - target[sand]) ** 2, axis=1)))


def with_params(scene, tan=None, cap=None, perm=None):
    """A copy of scene with the tan friction angle set, and the capillary
    values / cd multiplied by cap / perm (float32 parameters)."""
    s = copy.deepcopy(scene)
    p = s.params
    if tan is not None:
        p.dem_tan_friction_angle = float(np.float32(tan))
    if cap is not None:
        p.sf_c0 = float(np.float32(scene.params.sf_c0 * cap))
        p.sf_cmc = float(np.float32(scene.params.sf_cmc * cap))
        p.sf_csat = float(np.float32(scene.params.sf_csat * cap))
    if perm is not None:
        p.sf_cd = float(np.float32(scene.params.sf_cd * perm))
        sand = scene.label == SF_LABEL_SAND
        s.cda0asat[sand, 0] = (scene.cda0asat[sand, 0] * np.float32(perm)).astype(np.float32)
    return s


def directional_state(oracle_mod, scene, dt, n_sub, target, which, u, h):
    """(L(s + h u) - L(s - h u)) / 2h for s = initial positions or velocities."""
    base = (scene.pos if which == "pos" else scene.vel).astype(np.float64)
    lp = loss(oracle_mod, scene, dt, n_sub, target, **{which: base + h * u})
    lm = loss(oracle_mod, scene, dt, n_sub, target, **{which: base - h * u})
    return (lp - lm) / (2.0 * h)


def param_derivative(oracle_mod, scene, dt, n_sub, target, which, h):
    """dL/d tan friction angle, capillary scale or permeability scale."""
    if which == "tan":
        t0 = scene.params.dem_tan_friction_angle
        tp, tm = float(np.float32(t0 + h)), float(np.float32(t0 - h))
        lp = loss(oracle_mod, with_params(scene, tan=tp), dt, n_sub, target)
        lm = loss(oracle_mod, with_params(scene, tan=tm), dt, n_sub, target)
        return (lp - lm) / (tp - tm)
    lp = loss(oracle_mod, with_params(scene, **{which: 1.0 + h}), dt, n_sub, target)
    lm = loss(oracle_mod, with_params(scene, **{which: 1.0 - h}), dt, n_sub, target)
    return (lp - lm) / (2.0 * h)


# step sizes (coarse, fine) per direction; the two must agree before the FD is used
STEPS = {"pos": (1e-6, 1e-7), "vel": (1e-4, 1e-5), "tan": (2.0 ** -8, 2.0 ** -10),
         "cap": (2.0 ** -8, 2.0 ** -10), "perm": (2.0 ** -8, 2.0 ** -10)}


def checked_fd(fn, steps, consistency):
    """FD at two step sizes; fails when they disagree (the loss is not smooth
    enough along this direction for FD to be a reference)."""
    a, b = fn(steps[0]), fn(steps[1])
    rel = abs(a - b) / max(abs(b), 1e-300)
    assert rel <= consistency, f"finite differences not converged: {a:.9e} vs {b:.9e} (rel {rel:.2e})"
    return b


def jvp(oracle_mod, scene, dt, n_sub, target, which, u=None) -> float:
    """Exact pathwise directional derivative of the loss from the FP64
    forward-mode oracle: along u for which = "pos" / "vel", or by the
    parameter which = "tan" / "cap" / "perm"."""
    o = oracle_mod.Oracle(scene, precision=65)
    if which in ("pos", "vel"):
        o.set_tangent(which, u)   # creation order before the first sort
    else:
        o.seed_param(which)
    o.substeps(dt, False, n_sub)
    p = o.field("pos")
    t = o.tangent("pos")
    ids = o.field("id").astype(np.int64)
    x = np.empty_like(p)
    dx = np.empty_like(t)
    x[ids] = p
    dx[ids] = t
    sand = scene.label == SF_LABEL_SAND
    return float(np.mean(np.sum(2.0 * (x[sand] - target[sand]) * dx[sand], axis=1)))

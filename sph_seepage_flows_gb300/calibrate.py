"""Batched calibration of per-scene friction, capillary strength and
permeability by gradient descent through the adjoint.

Every iteration resets all scenes of one batched handle to their initial
state, applies each scene's parameters theta = (tan friction angle,
capillary scale, permeability scale), and runs one batched sf_adjoint_run:
n_substeps forward, then the reverse sweep, giving each scene's loss
mean_sand |x_T - target|^2 and its gradient. Adam then updates every scene's
theta independently.

    python -m sph_seepage_flows_gb300.calibrate [--scenes 32] [--substeps 500]
        [--checkpoint 25] [--iterations 50] [--lr 0.02]

runs the batched calibration workload: seeded column-collapse and
embankment-seepage scenes of 10k-50k particles whose targets are forward runs
with seeded per-scene parameters within +-10% of the reference values.
"""

from __future__ import annotations

import argparse
import copy
import json
import time

import numpy as np

from .params import SF_LABEL_SAND, reference_dt

THETA_NAMES = ("tan_friction_angle", "capillary_scale", "permeability_scale")


def scene_params(base, theta):
    """sf_params of a scene at theta (capillary values and cd scaled)."""
    p = copy.deepcopy(base.params)
    p.dem_tan_friction_angle = float(np.float32(theta[0]))
    p.sf_c0 = float(np.float32(base.params.sf_c0 * theta[1]))
    p.sf_cmc = float(np.float32(base.params.sf_cmc * theta[1]))
    p.sf_csat = float(np.float32(base.params.sf_csat * theta[1]))
    p.sf_cd = float(np.float32(base.params.sf_cd * theta[2]))
    return p


def apply_theta(sim, s, base, theta):
    """Parameters of scene s at theta, including the per-particle cd of MULTI scenes."""
    sim.set_params(scene_params(base, theta), scene=s)
    cda = base.cda0asat.copy()
    sand = base.label == SF_LABEL_SAND
    cda[sand, 0] = (base.cda0asat[sand, 0] * np.float32(theta[2])).astype(np.float32)
    sim.set_field("cda0asat", cda, order="id", scene=s)


def reset_state(sim, s, base):
    """Scene s back to its initial positions and velocities. Call
    sim.reset_order() first so that the run repeats a fresh handle's (the
    sort breaks ties within a cell by the order it finds)."""
    sim.set_field("pos", base.pos, order="id", scene=s)
    sim.set_field("vel", base.vel, order="id", scene=s)


def forward_targets(scenes, thetas, dt, n_substeps):
    """Final positions of a batched forward run at the given parameters."""
    from .capi import Simulation
    sim = Simulation(scenes)
    for s, (sc, th) in enumerate(zip(scenes, thetas)):
        apply_theta(sim, s, sc, th)
    sim.substeps_fixed(dt, n_substeps)
    out = [sim.field("pos", order="id", scene=s).astype(np.float32) for s in range(len(scenes))]
    sim.close()
    return out


class Adam:
    def __init__(self, shape, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.m = np.zeros(shape)
        self.v = np.zeros(shape)
        self.t = 0
        self.lr, self.b1, self.b2, self.eps = lr, beta1, beta2, eps

    def step(self, x, g):
        self.t += 1
        self.m = self.b1 * self.m + (1 - self.b1) * g
        self.v = self.b2 * self.v + (1 - self.b2) * g * g
        mh = self.m / (1 - self.b1 ** self.t)
        vh = self.v / (1 - self.b2 ** self.t)
        return x - self.lr * mh / (np.sqrt(vh) + self.eps)


# Seed scales of the adjoint (sf_set_adjoint_seed_scale). Over 500 substeps
# the workload's gradients reach 1e22-1e29 and the reverse sweep's
# intermediate products overflow FP32 (inf - inf gives NaN) for a changing
# few scenes per iteration, so every scene is seeded 2^-40 smaller from the
# start; a scene whose gradient is still not finite is seeded 2^-40 smaller
# again from the next iteration on (powers of two change no rounding), down
# to 2^-100, above which a seed of ~1e-3 stays clear of the subnormal range.
INITIAL_SEED_SCALE = 2.0 ** -40
SEED_STEP = 2.0 ** -40
SEED_FLOOR = 2.0 ** -100


def next_seed_scales(scales, finite):
    """Seed scales for the next iteration: scenes without a finite gradient
    this iteration get SEED_STEP times theirs (not below SEED_FLOOR)."""
    out = np.asarray(scales, dtype=np.float64).copy()
    bad = ~np.asarray(finite, dtype=bool)
    out[bad] = np.maximum(out[bad] * SEED_STEP, SEED_FLOOR)
    return out


def calibrate(scenes, targets, theta0, dt, n_substeps, checkpoint_every, iterations, lr=0.02,
              relative_step=True, callback=None, autotune=True):
    """Adam on every scene's theta; returns the loss / theta history and the
    device milliseconds of each batched adjoint run. With relative_step the
    update acts on log theta (steps relative to each parameter's size). A
    scene whose gradient is not finite keeps its theta that iteration and is
    seeded smaller from then on (next_seed_scales)."""
    from .capi import Simulation
    sim = Simulation(scenes)
    if autotune:
        sim.autotune(dt)
    theta = np.array(theta0, dtype=np.float64).reshape(len(scenes), 3)
    target = np.concatenate([np.asarray(t, np.float32).reshape(-1, 3) for t in targets])
    opt = Adam(theta.shape, lr)
    history = {"loss": [], "theta": [], "ms": [], "seed_scale": []}
    scales = np.full(len(scenes), INITIAL_SEED_SCALE)
    for it in range(iterations):
        sim.reset_order()
        for s, sc in enumerate(scenes):
            reset_state(sim, s, sc)
            apply_theta(sim, s, sc, theta[s])
            sim.set_adjoint_seed_scale(float(scales[s]), scene=s)
        t0 = time.perf_counter()
        res = sim.adjoint(dt, n_substeps, target, checkpoint_every=checkpoint_every, want_state_grads=False)
        wall = time.perf_counter() - t0
        # gradients of a factor on the current value -> gradients in theta
        g = res["grad_params"].astype(np.float64)
        g[:, 1] /= theta[:, 1]
        g[:, 2] /= theta[:, 2]
        # a scene whose gradient overflowed (exponential growth of the
        # cotangents over long horizons) keeps its theta this iteration
        bad = ~np.all(np.isfinite(g), axis=1)
        g[bad] = 0.0
        history.setdefault("nonfinite_gradients", []).append(int(bad.sum()))
        history["seed_scale"].append(scales.tolist())
        scales = next_seed_scales(scales, ~bad)
        history["loss"].append(res["loss"].astype(np.float64).tolist())
        history["theta"].append(theta.tolist())
        history["ms"].append({"forward": res["ms_forward"], "reverse": res["ms_reverse"], "wall": 1e3 * wall})
        if callback:
            callback(it, res, theta)
        if relative_step:
            theta = np.exp(opt.step(np.log(theta), g * theta))
        else:
            theta = opt.step(theta, g)
    sim.close()
    history["theta_final"] = theta.tolist()
    return history


def workload(n_scenes=32, seed=77, perturb=0.1):
    """The calibration scenes, the reference theta and seeded true thetas."""
    from . import scenes as S
    scs = S.calibration_scenes(n_scenes=n_scenes, seed=seed)
    theta0 = np.array([[sc.params.dem_tan_friction_angle, 1.0, 1.0] for sc in scs])
    rng = np.random.default_rng(seed + 1)
    theta_true = theta0 * (1.0 + rng.uniform(-perturb, perturb, size=theta0.shape))
    dt = reference_dt(scs[0].params, scs[0].bparams, scs[0].sparams)[1]
    return scs, theta0, theta_true, dt


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scenes", type=int, default=32)
    ap.add_argument("--substeps", type=int, default=500)
    ap.add_argument("--checkpoint", type=int, default=25)
    ap.add_argument("--iterations", type=int, default=50)
    ap.add_argument("--lr", type=float, default=0.02)
    ap.add_argument("--seed", type=int, default=77)
    args = ap.parse_args()
    scs, theta0, theta_true, dt = workload(args.scenes, args.seed)
    targets = forward_targets(scs, theta_true, dt, args.substeps)
    h = calibrate(scs, targets, theta0, dt, args.substeps, args.checkpoint, args.iterations, args.lr)
    loss = np.array(h["loss"])
    ms = h["ms"]
    out = {"scenes": len(scs), "particles": int(sum(s.n for s in scs)), "substeps": args.substeps,
           "checkpoint_every": args.checkpoint, "iterations": args.iterations, "dt": dt,
           "loss_first_mean": float(loss[0].mean()), "loss_last_mean": float(loss[-1].mean()),
           "scenes_improved": int((loss[-1] < loss[0]).sum()),
           "ms_per_iteration_device": float(np.median([m["forward"] + m["reverse"] for m in ms])),
           "ms_per_iteration_wall": float(np.median([m["wall"] for m in ms])),
           "theta_error_first": float(np.abs(np.array(h["theta"][0]) / theta_true - 1).mean()),
           "theta_error_last": float(np.abs(np.array(h["theta_final"]) / theta_true - 1).mean())}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()

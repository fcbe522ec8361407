"""Reverse-mode adjoint of the GPU substep (sf_adjoint_run) against FP64
central finite differences of the oracle.

Tolerance: each directional derivative and each parameter derivative is
within 1e-3 relative of the FP64 finite difference (the gradient accuracy
the adjoint is built to). The FD references are checked for convergence at
two step sizes here and in test_adjoint_fd_cpu.py. Exact properties:
checkpointing changes nothing (bit-identical results for checkpoint
intervals 1, 3 and 8), the handle ends on the same state as
sf_substeps_fixed, and a batched handle gives each scene the results of a
single-scene handle. A torch.autograd.Function wrapping the C ABI checks
that the gradients compose with autograd.
"""

import numpy as np
import pytest

from fd_oracle import (DT, PROBE_CASES, STEPS, checked_fd, directional_state, loss, param_derivative,
                       probe_direction, probe_scene, probe_target)

pytestmark = pytest.mark.gpu

TOL = 1e-3
PARAMS = ("tan", "cap", "perm")


def sim_of(scene):
    from sph_seepage_flows_gb300.capi import Simulation
    return Simulation(scene)


@pytest.fixture(scope="module")
def runs(cuda_lib):
    out = {}
    for seed, n_sub, damping in PROBE_CASES:
        sc = probe_scene(seed, damping)
        sim = sim_of(sc)
        out[(seed, n_sub, damping)] = (sc, sim.adjoint(DT, n_sub, probe_target(sc), checkpoint_every=1))
        sim.close()
    return out


@pytest.mark.parametrize("case", PROBE_CASES)
def test_loss_matches_oracle(runs, oracle_mod, case):
    sc, res = runs[case]
    ref = loss(oracle_mod, sc, DT, case[1], probe_target(sc))
    assert abs(res["loss"][0] - ref) <= 1e-4 * ref


@pytest.mark.parametrize("case", PROBE_CASES)
@pytest.mark.parametrize("which", ["pos", "vel"])
def test_state_gradient_directional(runs, oracle_mod, case, which):
    sc, res = runs[case]
    u = probe_direction(sc, case[0])
    fd = checked_fd(lambda h: directional_state(oracle_mod, sc, DT, case[1], probe_target(sc), which, u, h),
                    STEPS[which], 1e-5)
    g = res["grad_pos0" if which == "pos" else "grad_vel0"].astype(np.float64)
    ad = float(np.sum(g * u))
    assert abs(ad - fd) <= TOL * abs(fd), (ad, fd)


@pytest.mark.parametrize("case", PROBE_CASES)
@pytest.mark.parametrize("k", range(3))
def test_parameter_gradient(runs, oracle_mod, case, k):
    sc, res = runs[case]
    fd = checked_fd(lambda h: param_derivative(oracle_mod, sc, DT, case[1], probe_target(sc), PARAMS[k], h),
                    STEPS[PARAMS[k]], 1e-4)
    ad = float(res["grad_params"][0, k])
    assert abs(ad - fd) <= TOL * abs(fd), (PARAMS[k], ad, fd)


def test_gradient_is_not_trivial(runs):
    """Every tested derivative is well away from zero (the comparisons above
    would pass vacuously otherwise)."""
    sc, res = runs[PROBE_CASES[0]]
    assert np.all(np.abs(res["grad_params"][0]) > 1e-12)
    assert np.linalg.norm(res["grad_pos0"]) > 1e-3 and np.linalg.norm(res["grad_vel0"]) > 1e-7


def test_checkpointing_is_exact(cuda_lib):
    sc = probe_scene(11, 0.4)
    target = probe_target(sc)
    outs = []
    for k in (1, 3, 8):
        sim = sim_of(sc)
        r = sim.adjoint(DT, 8, target, checkpoint_every=k)
        r["final_pos"] = sim.field("pos", order="id")
        r["final_vel"] = sim.field("vel", order="id")
        outs.append(r)
        sim.close()
    for r in outs[1:]:
        for key in ("loss", "grad_params", "grad_pos0", "grad_vel0", "final_pos", "final_vel"):
            assert np.array_equal(r[key], outs[0][key]), key
    sim = sim_of(sc)
    sim.substeps_fixed(DT, 8)
    assert np.array_equal(sim.field("pos", order="id"), outs[0]["final_pos"])
    assert np.array_equal(sim.field("vel", order="id"), outs[0]["final_vel"])


def test_batched_equals_single(cuda_lib):
    from sph_seepage_flows_gb300.capi import Simulation
    scs = [probe_scene(11, 0.4), probe_scene(12, 0.0)]
    targets = [probe_target(s) for s in scs]
    single = []
    for s, t in zip(scs, targets):
        sim = Simulation(s)
        single.append(sim.adjoint(DT, 8, t))
        sim.close()
    sim = Simulation(scs)
    both = sim.adjoint(DT, 8, np.concatenate(targets), checkpoint_every=4)
    n0 = scs[0].n
    for s, r in enumerate(single):
        sl = slice(0, n0) if s == 0 else slice(n0, None)
        assert both["loss"][s] == r["loss"][0]
        assert np.array_equal(both["grad_params"][s], r["grad_params"][0])
        assert np.array_equal(both["grad_pos0"][sl], r["grad_pos0"])
        assert np.array_equal(both["grad_vel0"][sl], r["grad_vel0"])


def test_argument_errors(cuda_lib):
    from sph_seepage_flows_gb300.capi import SfError
    sc = probe_scene(11, 0.4)
    sim = sim_of(sc)
    t = probe_target(sc)
    for kw in ({"dt": 0.0, "n_substeps": 4}, {"dt": DT, "n_substeps": 0}):
        with pytest.raises(SfError):
            sim.adjoint(kw["dt"], kw["n_substeps"], t)
    with pytest.raises(SfError):
        sim.adjoint(DT, 4, t, checkpoint_every=0)
    with pytest.raises(ValueError):
        sim.adjoint(DT, 4, t[:-1])


def test_autograd_function(cuda_lib):
    """The C ABI wrapped as a torch.autograd.Function (test harness only):
    backward of the loss returns the adjoint's gradients."""
    torch = pytest.importorskip("torch")
    sc = probe_scene(11, 0.4)

    class Rollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, v0, target):
            s = probe_scene(11, 0.4)
            s.pos = x0.detach().cpu().numpy().astype(np.float32)
            s.vel = v0.detach().cpu().numpy().astype(np.float32)
            sim = sim_of(s)
            r = sim.adjoint(DT, 8, target.detach().cpu().numpy())
            sim.close()
            ctx.save_for_backward(torch.from_numpy(r["grad_pos0"]), torch.from_numpy(r["grad_vel0"]))
            return torch.tensor(float(r["loss"][0]), dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            gx, gv = ctx.saved_tensors
            return g * gx.double(), g * gv.double(), None

    x0 = torch.tensor(sc.pos, dtype=torch.float64, requires_grad=True)
    v0 = torch.tensor(sc.vel, dtype=torch.float64, requires_grad=True)
    out = 3.0 * Rollout.apply(x0, v0, torch.tensor(probe_target(sc)))
    out.backward()
    sim = sim_of(sc)
    r = sim.adjoint(DT, 8, probe_target(sc))
    assert np.allclose(x0.grad.numpy(), 3.0 * r["grad_pos0"], rtol=1e-6, atol=0)
    assert np.allclose(v0.grad.numpy(), 3.0 * r["grad_vel0"], rtol=1e-6, atol=0)


def test_long_horizon_gradients_stay_finite(cuda_lib):
    """200 substeps of the 20k column, twice (the second run starts from a
    re-set state whose particles are in another slot order): the cotangents
    grow by orders of magnitude but no quotient-rule term may overflow to a
    non-finite value."""
    from sph_seepage_flows_gb300 import calibrate, scenes
    from sph_seepage_flows_gb300.params import reference_dt
    sc = scenes.adjoint_column()
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    target = calibrate.forward_targets([sc], [np.array([sc.params.dem_tan_friction_angle, 1.1, 1.1])], dt, 200)[0]
    sim = sim_of(sc)
    for _ in range(2):
        r = sim.adjoint(dt, 200, target)
        for key in ("loss", "grad_params", "grad_pos0", "grad_vel0"):
            assert np.all(np.isfinite(r[key])), key
        calibrate.reset_state(sim, 0, sc)


def test_seed_scale_changes_no_gradient_bit(cuda_lib):
    """sf_set_adjoint_seed_scale with a power of two: every cotangent of the
    reverse sweep is scaled exactly, so after the scale is divided out the
    gradients equal the unscaled run's bit for bit; sf_set_params keeps it."""
    sc = probe_scene(11, 0.4)
    target = probe_target(sc)
    outs = []
    for scale in (1.0, 2.0 ** -20, 2.0 ** 12):
        sim = sim_of(sc)
        sim.set_adjoint_seed_scale(scale)
        sim.set_params(sc.params)
        outs.append(sim.adjoint(DT, 8, target, checkpoint_every=4))
        sim.close()
    for r in outs[1:]:
        for key in ("loss", "grad_params", "grad_pos0", "grad_vel0"):
            assert np.array_equal(r[key], outs[0][key]), key
    from sph_seepage_flows_gb300.capi import SfError
    sim = sim_of(sc)
    for bad in (0.0, -1.0, float("inf"), float("nan")):
        with pytest.raises(SfError):
            sim.set_adjoint_seed_scale(bad)
    sim.close()


def test_reset_order_repeats_a_fresh_run(cuda_lib):
    """sf_reset_order puts the particles back in creation order: a gradient
    run from positions and velocities reset by id then repeats a fresh
    handle's run bit for bit (the first sort breaks ties within a cell by
    the order it finds, and that order sets the FP32 order of every sum)."""
    from sph_seepage_flows_gb300 import calibrate, scenes
    from sph_seepage_flows_gb300.params import reference_dt
    sc = scenes.tiny(seed=7)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    target = calibrate.forward_targets([sc], [np.array([sc.params.dem_tan_friction_angle, 1.1, 1.1])], dt, 16)[0]
    fresh = sim_of(sc)
    ref = fresh.adjoint(dt, 16, target, checkpoint_every=8)
    fresh.close()
    sim = sim_of(sc)
    sim.substeps_fixed(dt, 40)  # the particles move and the order changes
    assert not np.array_equal(sim.field("id"), np.arange(sc.n, dtype=np.int32))
    sim.reset_order()
    assert np.array_equal(sim.field("id"), np.arange(sc.n, dtype=np.int32))
    calibrate.reset_state(sim, 0, sc)
    r = sim.adjoint(dt, 16, target, checkpoint_every=8)
    for key in ("loss", "grad_params", "grad_pos0", "grad_vel0"):
        assert np.array_equal(r[key], ref[key]), key
    sim.close()


def test_reset_order_in_a_batched_handle(cuda_lib):
    """sf_reset_order in a handle of several scenes: each scene's particles go
    back to creation order within its own slots, and substeps from a state
    reset by id equal a fresh handle's bit for bit."""
    from sph_seepage_flows_gb300 import calibrate, scenes
    from sph_seepage_flows_gb300.capi import Simulation
    from sph_seepage_flows_gb300.params import reference_dt
    sc = [scenes.tiny(seed=3), scenes.tiny(seed=4, sand=(6, 6, 6), water=(4, 4, 4))]
    dt = reference_dt(sc[0].params, sc[0].bparams, sc[0].sparams)[1]
    fresh = Simulation(sc)
    fresh.substeps_fixed(dt, 10)
    sim = Simulation(sc)
    sim.substeps_fixed(dt, 30)
    sim.reset_order()
    for k, s in enumerate(sc):
        assert np.array_equal(sim.field("id", scene=k), np.arange(s.n, dtype=np.int32)), k
        calibrate.reset_state(sim, k, s)
    sim.substeps_fixed(dt, 10)
    for k in range(len(sc)):
        for name in ("pos", "vel", "density", "id"):
            assert np.array_equal(sim.field(name, scene=k), fresh.field(name, scene=k)), (k, name)
    sim.close()
    fresh.close()


def test_reset_order_after_added_particles(cuda_lib):
    """Particles added by sf_add_sph_particles take the next ids; after some
    substeps the order reset puts every particle, the added ones included,
    at the slot of its id, with its position and velocity."""
    from sph_seepage_flows_gb300 import scenes
    from sph_seepage_flows_gb300.capi import Simulation
    from sph_seepage_flows_gb300.params import reference_dt
    sc = scenes.tiny(seed=5)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    sim = Simulation(sc, capacity=sc.n + 64)
    sim.substeps_fixed(dt, 4)
    pts = np.array([[0.2, 0.34, 0.2], [0.22, 0.34, 0.2], [0.2, 0.34, 0.22]], np.float32)  # above the material
    sim.add_sph_particles(pts, np.array([0.3, 0.6, 1.0], np.float32), np.array([0.0, -1.0, 0.0], np.float32),
                          sc.params.sph_mass, sc.params.sph_particle_radius)
    sim.substeps_fixed(dt, 20)
    n = sim.size()
    assert n == sc.n + 3
    pos_by_id, vel_by_id = sim.field("pos", order="id"), sim.field("vel", order="id")
    sim.reset_order()
    assert np.array_equal(sim.field("id"), np.arange(n, dtype=np.int32))
    assert np.array_equal(sim.field("pos"), pos_by_id)
    assert np.array_equal(sim.field("vel"), vel_by_id)
    sim.substeps_fixed(dt, 2)
    assert sim.check_error() == 0
    sim.close()

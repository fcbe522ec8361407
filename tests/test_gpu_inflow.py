"""Dynamic SPH inflow on the GPU (CudaSFSystem::OnUpdateSolver's emitter,
cuda_sf_system.cu:86-115, and CudaSFParticles::AddSphParticles,
cuda_sf_particles.cu:50-68).

tests/cpp/inflow_main.cpp runs the facade scene with a square emitter
switched on, under the WCSPH schedule (emit when |v| * elapsed / (2 r)
reaches the emission counter, elapsed summing render_interval / N_sub) and
the SPH schedule (every floor(2 r / (|v| dt)) calls), with 32 slots of
headroom (three emissions of the 9-point emitter) so that the capacity
cut-off switches the emitter off at the fourth. Checks:

* the facade program equals a Python run of the C ABI (sf_step +
  sf_add_sph_particles) under a restatement of the same schedule, call for
  call (particle counts) and bit for bit at the end;
* that run against the FP32 oracle (oracle AddSphParticles) one call at a
  time from identical inputs: sub-step counts, sorted ids, positions within
  1e-5 m and density within 1e-4 after every call, emissions included;
* where the reference's own CUDA library is built, its emitter and schedule
  give the same particle count after every call, and the particles it
  appends are the emitter points, bit for bit.
"""

import subprocess

import numpy as np
import pytest

from helpers import CARRIED, build_facade_program, facade_scene, rel_err
from sph_seepage_flows_gb300.params import SF_SOLVER_SPH

pytestmark = pytest.mark.gpu

T_FRAME = np.float32(1.0 / 30.0)
CALLS = {"wcsph": 130, "sph": 80}
EMITTER = {"pos": (0.2, 0.2, 0.2), "vel": (0.0, -1.0, 0.0), "col": (0.3, 0.6, 1.0), "type": "square",
           "radius": 0.03}
HEADROOM = 32


def read_dump(path):
    with open(path, "rb") as f:
        n0, npts, calls = np.frombuffer(f.read(24), np.int64)
        init = np.frombuffer(f.read(12 * n0), np.float32).reshape(n0, 3)
        points = np.frombuffer(f.read(12 * npts), np.float32).reshape(npts, 3)
        counts = np.frombuffer(f.read(8 * calls), np.int64)
        nsubs = np.frombuffer(f.read(8 * calls), np.int64)
        n = int(np.frombuffer(f.read(8), np.int64)[0])
        pos = np.frombuffer(f.read(12 * n), np.float32).reshape(n, 3)
        vel = np.frombuffer(f.read(12 * n), np.float32).reshape(n, 3)
    return {"init": init, "points": points, "counts": counts, "nsubs": nsubs, "pos": pos, "vel": vel}


class Schedule:
    """The emitter schedule of cuda_sf_system.cu:86-115 in float32."""

    def __init__(self, solver, params, npts, capacity):
        self.wcsph = solver == "wcsph"
        v = np.asarray(EMITTER["vel"], np.float32)
        self.speed = np.sqrt(np.float32(v @ v)).astype(np.float32)
        self.two_r = np.float32(2.0) * np.float32(params.sph_particle_radius)
        self.dt = np.float32(params.dt)
        self.npts, self.capacity = npts, capacity
        self.counter, self.elapsed, self.enabled = 0, np.float32(0.0), True

    def fire(self, nsub):
        if not self.enabled:
            return False
        if self.wcsph:
            self.elapsed = np.float32(self.elapsed + np.float32(T_FRAME / np.float32(nsub)))
            if np.float32(np.float32(self.speed * self.elapsed) / self.two_r) >= np.float32(self.counter):
                self.counter += 1
                return True
            return False
        step = int(np.float32(self.two_r / np.float32(self.speed * self.dt)))
        if step == 0:
            return True
        go = self.counter % step == 0
        self.counter += 1
        return go

    def admit(self, n):
        """Size() + emitted < MaxSize(), else the emitter switches off."""
        if n + self.npts < self.capacity:
            return True
        self.enabled = False
        return False


def scene_for(solver, init):
    sc = facade_scene(init)
    if solver == "sph":
        sc.params.solver_type = SF_SOLVER_SPH
    return sc


@pytest.fixture(scope="module")
def inflow_runs(cuda_lib, tmp_path_factory):
    tmp = tmp_path_factory.mktemp("inflow")
    exe = build_facade_program(tmp, "inflow_main")
    runs = {}
    for solver, calls in CALLS.items():
        dump = str(tmp / f"{solver}.bin")
        out = subprocess.run([exe, dump, solver, str(calls)], capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "inflow ok" in out.stdout and "emitter=0" in out.stdout, out.stdout
        runs[solver] = read_dump(dump)
    return runs


def python_run(run, solver, oracle_mod=None):
    """The C ABI under the restated schedule; with oracle_mod, the FP32
    oracle follows it one call at a time from the GPU's state."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scene_for(solver, run["init"])
    cap = sc.n + HEADROOM
    sim = Simulation(sc, capacity=cap)
    o32 = oracle_mod.Oracle(sc, 32) if oracle_mod else None
    sched = Schedule(solver, sc.params, len(run["points"]), cap)
    col = np.asarray(EMITTER["col"], np.float32)
    vel = np.asarray(EMITTER["vel"], np.float32)
    counts, worst = [], 0.0
    for _ in range(len(run["counts"])):
        nsub = sim.step(float(T_FRAME))
        if o32 is not None:
            o32.substeps(float(T_FRAME), True, 1)
            assert o32.num_substeps == nsub
            assert np.array_equal(sim.field("id"), o32.field("id").astype(np.int32))
            d = np.abs(sim.field("pos").astype(np.float64) - o32.field("pos")).max()
            worst = max(worst, float(d))
            assert d < 1e-5, d
            assert rel_err(sim.field("density"), o32.field("density")) < 1e-4
            for name in CARRIED:
                o32.set_field(name, sim.field(name))
        if sched.fire(nsub) and sched.admit(sim.size()):
            sim.add_sph_particles(run["points"], col, vel, sc.params.sph_mass, sc.params.sph_particle_radius)
            if o32 is not None:
                assert o32.add_sph_particles(run["points"], col, vel, sc.params.sph_mass,
                                             sc.params.sph_particle_radius, cap)
        counts.append(sim.size())
    return sim, np.array(counts), worst


@pytest.mark.parametrize("solver", ["wcsph", "sph"])
def test_facade_inflow_equals_c_abi_under_the_schedule(inflow_runs, solver):
    run = inflow_runs[solver]
    sim, counts, _ = python_run(run, solver)
    n0, npts = len(run["init"]), len(run["points"])
    assert np.array_equal(counts, run["counts"])
    emitted = (counts[-1] - n0) // npts
    assert emitted == 3 and counts[-1] + npts >= n0 + HEADROOM, (emitted, counts[-1])
    assert np.array_equal(sim.field("pos", order="id"), run["pos"])
    assert np.array_equal(sim.field("vel", order="id"), run["vel"])
    ids = sim.field("id", order="id")
    assert np.array_equal(ids, np.arange(counts[-1]))
    label = sim.field("label", order="id")
    assert (label[n0:] == 0).all()


@pytest.mark.parametrize("solver", ["wcsph", "sph"])
def test_inflow_tracks_oracle_call_by_call(inflow_runs, oracle_mod, solver):
    run = inflow_runs[solver]
    _, counts, worst = python_run(run, solver, oracle_mod)
    assert np.array_equal(counts, run["counts"])
    print(f"{solver}: {len(counts)} calls, {counts[-1] - counts[0]} emitted, max |dx| per call {worst:.2e} m")


@pytest.mark.parametrize("solver", ["wcsph", "sph"])
def test_inflow_matches_reference_gpu_schedule(inflow_runs, oracle_mod, solver):
    if oracle_mod.build_ref_gpu() is None:
        pytest.skip("the reference CUDA library is not staged here (oracle/build_ref_cuda.sh)")
    run = inflow_runs[solver]
    sc = scene_for(solver, run["init"])
    npts = len(run["points"])
    r = oracle_mod.RefGpu(sc, capacity=sc.n + HEADROOM, emitter=EMITTER)
    counts = []
    for k in range(len(run["counts"])):
        before = r.n
        r.update(float(T_FRAME))
        assert r.num_substeps == run["nsubs"][k], k
        counts.append(r.n)
        if r.n > before:
            # AddSphParticles appends after the live particles: the emitter points
            tail = r.field("pos")[before:].astype(np.float32)
            assert r.n - before == npts
            assert np.array_equal(tail, run["points"]), k
    assert np.array_equal(np.array(counts), run["counts"])

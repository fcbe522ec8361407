"""Benchmark of the coupled SPH-DEM seepage-flow substep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A step is one substep of the whole scene (sort + six neighbor passes +
integrate) at the reference dt, held fixed (the WCSPH CFL value at rest,
2.415e-4 s for h = 0.02). Default workload: the 1M-particle embankment scene
(~500k DEM sand, r = 0.005, + ~500k WCSPH water, pitch 0.01; seeded synthetic
geometry). The metric is particle-substeps/s (whole job).

Printed JSON line (rank 0): value = device-resident throughput from CUDA
events around K steps (graph-replayed); e2e = the same metric through the C ABI
with host buffers (each step copies positions and velocities in from pinned
host memory, runs the substep, and copies them back); roofline of the dominant
kernel from per-stage CUDA-event timings against the measured HBM peak;
cpu_baseline = the FP32 CPU oracle (all host threads) on a bounded sample.

--impl reference times the reference's CPU implementation of the path: the
reference has no CPU physics, so this is the FP32 CPU restatement of its
kernels (oracle/, pinned bit-exact to the reference kernels), on all host
threads, one substep of the same scene per step.

Also reported (same GPU, device time): "batched", the 64-scene ensemble in
one handle against a loop of per-scene handles; "adjoint", the 20k-particle
column over 200 substeps, gradient run (sf_adjoint_run) against a forward run;
"calibration", per-iteration time of the 32-scene batched Adam calibration.

Multi-GPU: scenes are independent replicas (no collective); under torchrun
every rank runs its own copy and value = sum over ranks (weak scaling).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per particle-substep of each stage: the reference pass
# sequence with every array read and written once per pass (4 B scalars,
# 12 B vectors), neighbour gathers counted once.
STAGE_BYTES = {
    "sort": 16 + 148 + 5,          # hash + sort/reorder + cell count/scan
    "density": 24 + 12,            # density + pressure
    "avgflow": 56,
    "voidage_adhesion": 32 + 52 + 40,  # sand voidage + water adhesion + wet colour
    "sand_momentum": 112 + 6,      # + half of extra forces
    "water_momentum": 92 + 6 + 12,  # + half of extra forces + CFL max
    "integrate": 64 + 52 + 24,     # integrate + water clamp + adhesion clears
}
BYTES_PER_SUBSTEP = sum(STAGE_BYTES.values())  # 753

# DRAM bytes (read + write) per launch of each stage's main kernel on the 1M
# workload, from one ncu capture, tagged with the digest of the sources that
# kernel is compiled from (its translation unit and the headers it includes,
# csrc_digest(KERNEL_SOURCES[stage])) at the capture. When those sources have
# changed since, the figure no longer describes the running kernel and is
# reported as null.
KERNEL_SOURCES = {"density": ("sf_kernels.cu", "sf_kernels.h", "sf_device.cuh", "sf_neighbors.cuh")}
NCU_TRAFFIC = {"density": (282.0e6, "0abe114f76e1")}


def roofline_traffic(stage: str, workload: str):
    """(DRAM bytes per launch, where they come from) of the stage's kernel on
    the 1M workload, or (None, why) when no capture describes its current
    sources."""
    if workload != "plain_large" or stage not in NCU_TRAFFIC:
        return None, "no ncu capture of this kernel on this workload"
    digest = csrc_digest(KERNEL_SOURCES.get(stage))
    if digest != NCU_TRAFFIC[stage][1]:
        return None, "no ncu capture of the current kernel sources"
    return NCU_TRAFFIC[stage][0], f"ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, kernel sources {digest}"


def csrc_digest(names=None) -> str:
    """sha256 (first 12 hex digits) of the named CUDA sources (default: all),
    in name order."""
    import hashlib
    d = hashlib.sha256()
    csrc = os.path.join(ROOT, "sph_seepage_flows_gb300", "csrc")
    for name in sorted(names or os.listdir(csrc)):
        if name.endswith((".cu", ".cuh", ".h")):
            with open(os.path.join(csrc, name), "rb") as f:
                d.update(name.encode() + b"\0" + f.read())
    return d.hexdigest()[:12]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_scene(name: str):
    from sph_seepage_flows_gb300 import scenes
    if name == "plain_large":
        return scenes.plain_large()
    if name == "plain_small":
        return scenes.plain_small()
    if name == "tiny":
        return scenes.tiny()
    if name == "column":  # the 20k sand column of the adjoint workload
        return scenes.adjoint_column()
    raise SystemExit(f"unknown workload {name}")


def reference_dt(sc):
    from sph_seepage_flows_gb300.params import reference_dt as rdt
    return rdt(sc.params, sc.bparams, sc.sparams)[1]


def cpu_baseline(sc, dt, budget_s=20.0):
    """FP32 oracle (all host threads) on the same scene: one warm-up substep,
    then substeps until budget_s of CPU work."""
    import oracle
    threads = oracle.set_threads(os.cpu_count() or 1)
    o = oracle.Oracle(sc, 32)
    t0 = time.perf_counter()
    o.substeps(dt, False, 1)
    first = time.perf_counter() - t0
    n = max(1, min(20, int(budget_s / max(first, 1e-3))))
    t0 = time.perf_counter()
    o.substeps(dt, False, n)
    el = time.perf_counter() - t0
    return {"value": sc.n * n / el, "unit": "particle-substeps/s", "cores": threads, "kind": "port",
            "sample": f"{n} substeps of the full {sc.n}-particle scene after 1 warm-up substep "
                      f"(FP32 CPU restatement of the reference kernels, OpenMP)"}


def reference_gpu_baseline(sc, calls=10):
    """The reference's own CUDA library on the same GPU: seepage_flows_cuda
    built for sm_103a with its own -use_fast_math flags
    (oracle/build_ref_cuda.sh) and driven through its public classes
    (oracle/ref_gpu_driver.cu). Each step is one
    CudaBaseSystem::UpdateSystem(1/30 s) call on the same scene: one substep
    of (1/30) / N_sub = the reference dt at rest, ending, as the reference
    does, with a device synchronisation. Wall time of `calls` calls after one
    warm-up call (CUDA events around them)."""
    import oracle
    try:
        if oracle.build_ref_gpu() is None:
            return {"unavailable": "reference CUDA sources not staged (oracle/build_ref_cuda.sh)"}
    except Exception as e:  # noqa: BLE001 - a baseline leg reports, never aborts the bench
        return {"unavailable": f"reference CUDA build failed: {e}"[:300]}
    import torch
    r = oracle.RefGpu(sc)
    T = 1.0 / 30.0
    r.update(T)
    torch.cuda.nvtx.range_push("reference_gpu")  # lets a profiler capture exactly the timed calls
    ms = r.run(T, calls)
    torch.cuda.nvtx.range_pop()
    nsub = r.num_substeps
    del r
    return {"value": sc.n * calls / (ms * 1e-3), "unit": "particle-substeps/s", "ms_per_substep": ms / calls,
            "calls": calls, "n_sub": nsub, "dt": T / nsub,
            "path": "reference seepage_flows_cuda (-use_fast_math, sm_103a): CudaSFSystem::UpdateSystem(1/30 s)"}


def batched_comparison(stream, substeps=100, n_scenes=64, blocks=10):
    """The batched-ensemble workload: n_scenes independent scenes (log-uniform
    2k-60k particles, per-scene friction/capillary/permeability) advanced in
    the same launches by one handle, against a loop over one handle per scene
    on the same GPU, for the ensemble's 1000 substeps (10 blocks of 100). Both
    replay captured graphs of `substeps`-substep blocks (graph capture covers
    two substeps; a block is substeps/2 replays)."""
    import torch

    from sph_seepage_flows_gb300 import capi, scenes
    sc = scenes.batched(n_scenes=n_scenes)
    dt = reference_dt(sc[0])
    total = sum(s.n for s in sc)
    batch = capi.Simulation(sc, stream=stream.cuda_stream)
    singles = [capi.Simulation(s, stream=stream.cuda_stream) for s in sc]
    batch.substeps_fixed(dt, 4)
    for s in singles:
        s.substeps_fixed(dt, 4)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(blocks):
        batch.substeps_fixed(dt, substeps)
    e1.record(stream)
    torch.cuda.synchronize()
    t_batch = e0.elapsed_time(e1) / 1e3
    e0.record(stream)
    for _ in range(blocks):
        for s in singles:
            s.substeps_fixed(dt, substeps)
    e1.record(stream)
    torch.cuda.synchronize()
    t_loop = e0.elapsed_time(e1) / 1e3
    flags = batch.check_error()
    for s in singles:
        flags |= s.check_error()
    v_batch = total * substeps * blocks / t_batch
    v_loop = total * substeps * blocks / t_loop
    return {"scenes": n_scenes, "particles": total, "substeps": substeps * blocks, "dt": dt,
            "batched_value": v_batch, "per_scene_loop_value": v_loop, "speedup": v_batch / v_loop,
            "unit": "particle-substeps/s", "device_error_flags": flags}


def adjoint_comparison(stream, n_substeps=200, checkpoint_every=20):
    """The adjoint workload: the 20k-particle sand column collapsing for
    n_substeps at the reference dt; loss = mean squared distance of the final
    sand positions to a forward run with tan friction angle, capillary and
    permeability scales +10%. Gradient run (sf_adjoint_run: forward with
    checkpoints + reverse sweep) against a plain forward run of the same
    substeps, both device-timed."""
    import torch

    from sph_seepage_flows_gb300 import calibrate, capi, scenes
    sc = scenes.adjoint_column()
    dt = reference_dt(sc)
    theta0 = np.array([sc.params.dem_tan_friction_angle, 1.0, 1.0])
    target = calibrate.forward_targets([sc], [theta0 * 1.1], dt, n_substeps)[0]
    fwd = capi.Simulation(sc, stream=stream.cuda_stream)
    tuning = fwd.autotune(dt)
    fwd.substeps_fixed(dt, 2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fwd.substeps_fixed(dt, n_substeps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_fwd = e0.elapsed_time(e1)
    fwd.close()
    out = {"workload": "adjoint_column", "particles": sc.n, "substeps": n_substeps, "dt": dt,
           "forward_ms": ms_fwd, "tuning": tuning, "runs": {}}
    for k in (checkpoint_every, n_substeps):
        sim = capi.Simulation(sc, stream=stream.cuda_stream)
        sim.autotune(dt)
        sim.adjoint(dt, n_substeps, target, checkpoint_every=k, want_state_grads=False)  # allocates
        sim.reset_order()  # the timed run repeats a fresh handle's
        calibrate.reset_state(sim, 0, sc)
        r = sim.adjoint(dt, n_substeps, target, checkpoint_every=k)
        sim.close()
        out["runs"][str(k)] = {
            "checkpoint_every": k, "forward_ms": r["ms_forward"], "reverse_ms": r["ms_reverse"],
            "gradient_run_vs_forward": (r["ms_forward"] + r["ms_reverse"]) / ms_fwd,
            "reverse_vs_forward": r["ms_reverse"] / ms_fwd,
            "loss": float(r["loss"][0]), "grad_params": [float(v) for v in r["grad_params"][0]],
            "grad_vel0_norm": float(np.linalg.norm(r["grad_vel0"]))}
    return out


def adjoint_workload(args):
    """--adjoint-substeps K: the gradient run on the bench workload alone (K
    substeps, every substep stored unless --checkpoint-every is smaller),
    forward and reverse device time per substep against the graph-replayed
    forward; used for the ncu launch lists of the adjoint kernels (the second
    gradient run is bracketed by the NVTX range "timed")."""
    import torch

    from sph_seepage_flows_gb300 import capi
    sc = make_scene(args.workload)
    dt = reference_dt(sc)
    k = args.adjoint_substeps
    sim = capi.Simulation(sc)
    sim.autotune(dt)
    target = sc.pos.astype(np.float32) + np.float32(1e-3)
    ck = args.checkpoint_every if args.checkpoint_every > 0 else k
    sim.adjoint(dt, k, target, checkpoint_every=ck, want_state_grads=False)  # allocates and captures
    torch.cuda.nvtx.range_push("timed")
    r = sim.adjoint(dt, k, target, checkpoint_every=ck, want_state_grads=False)
    torch.cuda.nvtx.range_pop()
    stream = torch.cuda.Stream()
    fwd = capi.Simulation(sc, stream=stream.cuda_stream)
    fwd.substeps_fixed(dt, 2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fwd.substeps_fixed(dt, k)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    print(json.dumps({"adjoint_workload": args.workload, "particles": sc.n, "substeps": k, "checkpoint_every": ck,
                      "forward_ms_per_substep": ms / k, "store_forward_ms_per_substep": r["ms_forward"] / k,
                      "reverse_ms_per_substep": r["ms_reverse"] / k,
                      "gradient_run_vs_forward": (r["ms_forward"] + r["ms_reverse"]) / ms}), flush=True)


def calibration_timing(stream, iterations=2, n_substeps=500, checkpoint_every=25):
    """Per-iteration time of the batched calibration workload (32 scenes of
    10k-50k particles, 500 substeps, checkpoints every 25): `iterations`
    Adam iterations of one batched adjoint launch each."""
    from sph_seepage_flows_gb300 import calibrate
    scs, theta0, theta_true, dt = calibrate.workload()
    targets = calibrate.forward_targets(scs, theta_true, dt, n_substeps)
    # one untimed iteration first: it allocates the stored substeps and
    # captures the store-mode and reverse substep graphs
    h = calibrate.calibrate(scs, targets, theta0, dt, n_substeps, checkpoint_every, iterations + 1)
    ms = h["ms"][1:]
    return {"scenes": len(scs), "particles": int(sum(s.n for s in scs)), "substeps": n_substeps,
            "checkpoint_every": checkpoint_every, "iterations_timed": iterations, "warmup_iterations": 1,
            "device_ms_per_iteration": float(np.median([m["forward"] + m["reverse"] for m in ms])),
            "wall_ms_per_iteration": float(np.median([m["wall"] for m in ms])),
            "particle_substeps_per_s_forward_and_reverse":
                float(sum(s.n for s in scs) * n_substeps / (np.median([m["forward"] + m["reverse"] for m in ms]) * 1e-3)),
            "loss_mean_by_iteration": [float(np.mean(l)) for l in h["loss"]],
            "nonfinite_gradient_scenes_by_iteration": h.get("nonfinite_gradients", [])}


def long_run(stream, workload="plain_large", substeps=2000, window=200):
    """The whole configured run of the workload: `substeps` graph-replayed
    substeps at the reference dt from the initial state, timed per window of
    `window` substeps (CUDA events on the library's stream). The state
    evolves (the seepage front advances and the neighbour lists grow), so
    later windows cost more than the first; the list capacity is read after
    each window."""
    import torch

    from sph_seepage_flows_gb300 import capi
    sc = make_scene(workload)
    dt = reference_dt(sc)
    sim = capi.Simulation(sc, stream=stream.cuda_stream)
    tuning = sim.autotune(dt)
    windows = []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    total_ms = 0.0
    for w in range(substeps // window):
        ev[0].record(stream)
        sim.substeps_fixed(dt, window)
        ev[1].record(stream)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1])
        total_ms += ms
        cap, growths = sim.list_capacity()
        windows.append({"substeps": [w * window, (w + 1) * window], "ms_per_substep": ms / window,
                        "list_capacity": cap, "list_growths": growths})
    flags = sim.check_error()
    done = window * len(windows)
    sim.close()
    return {"workload": workload, "particles": sc.n, "substeps": done, "dt": dt,
            "mean_ms_per_substep": total_ms / done, "value": sc.n * done / (total_ms * 1e-3),
            "unit": "particle-substeps/s", "windows": windows, "device_error_flags": flags,
            "list_capacity_initial": tuning["list_capacity"]}


def run_reference(args, rank, world):
    """--impl reference: the reference kernels' FP32 CPU restatement."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    sc = make_scene(args.workload)
    dt = reference_dt(sc)
    threads = oracle.set_threads(os.cpu_count() or 1)
    o = oracle.Oracle(sc, 32)
    for _ in range(args.warmup):
        o.substeps(dt, False, 1)
    t0 = time.perf_counter()
    o.substeps(dt, False, args.steps)
    el = time.perf_counter() - t0
    v = sc.n * args.steps / el
    line = {"metric": "particle-substeps/s at 1M SPH+DEM", "value": v, "unit": "particle-substeps/s",
            "impl": "reference", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "particles": sc.n, "sand": sc.n_sand, "water": sc.n_water,
                       "dt": dt, "substeps_per_step": 1},
            "cpu_baseline": {"value": v, "unit": "particle-substeps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} substeps of the full scene after {args.warmup} warm-up"},
            "e2e": {"value": v, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import torch

    from sph_seepage_flows_gb300 import build as b
    from sph_seepage_flows_gb300 import capi
    from sph_seepage_flows_gb300.params import STAGES

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    b.build_library()
    sc = make_scene(args.workload)
    dt = reference_dt(sc)
    stream = torch.cuda.Stream()
    sim = capi.Simulation(sc, stream=stream.cuda_stream)
    n = sc.n

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    tuning = sim.autotune(dt)  # list capacity and per-pass block sizes for this scene
    if args.density_staging != "auto":  # fixed form of the density pass (profiling)
        sim.set_density_staging(args.density_staging == "on")
        tuning.update(sim.tuning())
    # warm-up (also captures the two-substep graph)
    sim.substeps_fixed(dt, 2 * max(1, (args.warmup + 1) // 2))
    sim.synchronize()
    steps = args.steps + (args.steps % 2)  # graph replays come in pairs
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    l0 = sim.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")  # lets a profiler capture exactly the timed substeps
    e0.record(stream)
    sim.substeps_fixed(dt, steps)
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = sim.launches() - l0
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n * steps / (ms * 1e-3)

    # per-stage timing (eager launches, CUDA events on the launching stream)
    stage_ms = {s: 0.0 for s in STAGES}
    reps = max(2, min(10, args.steps))
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(STAGES) + 1)]
    for _ in range(reps):
        evs[0].record(stream)
        for k, s in enumerate(STAGES):
            sim.stage(s, dt, adaptive=False)
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
        for k, s in enumerate(STAGES):
            stage_ms[s] += evs[k].elapsed_time(evs[k + 1]) / reps
    top = max(stage_ms, key=stage_ms.get)
    peak, peak_kind = peaks()
    traffic, traffic_source = roofline_traffic(top, args.workload)
    achieved = STAGE_BYTES[top] * n / (stage_ms[top] * 1e-3) / 1e9

    # e2e through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hpos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        hvel = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        hp = hpos.numpy()
        hv = hvel.numpy()
        sim.field("pos", out=hp)
        sim.field("vel", out=hv)
        e2e_steps = max(2, min(args.steps, 20))

        inputs = {"pos": hp, "vel": hv}

        def e2e_step():
            sim.set_fields(inputs)
            sim.substeps_fixed(dt, 1)
            sim.get_fields(inputs)

        e2e_step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([el], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            el = float(t.item())
        e2e = {"value": world * n * e2e_steps / el, "unit": "particle-substeps/s",
               "h2d_bytes_per_step": 2 * 12 * n, "d2h_bytes_per_step": 2 * 12 * n,
               "path": "sf_set_fields(pos, vel; pinned host) + sf_substeps_fixed(1) + sf_get_fields(pos, vel)"}

    flags = sim.check_error()
    # pair interactions per substep: for every particle, the particles within
    # the interaction reach (itself excluded) times the neighbour passes it
    # takes part in (water: density, avg flow, adhesion, momentum; sand: avg
    # flow, voidage, momentum)
    nbrs = sim.field("neighbors").astype(np.int64) - 1
    lab = sim.field("label")
    pairs = int(4 * nbrs[lab == 0].sum() + 3 * nbrs[lab == 1].sum())
    bgeo = None if args.no_bgeo else bgeo_export_timing(sim, n)
    frame = None if args.no_frame else frame_timing(sim, n)
    batched = None if args.no_batched else batched_comparison(stream)
    adjoint = None if args.no_adjoint else adjoint_comparison(stream)
    calib = None if args.no_calibration else calibration_timing(stream)
    longrun = None if args.no_long_run else long_run(stream, args.workload)
    ref_gpu = None if (args.no_reference_gpu or rank != 0) else reference_gpu_baseline(sc)
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_baseline(sc, dt)
    line = {
        "metric": "particle-substeps/s at 1M SPH+DEM", "value": value, "unit": "particle-substeps/s",
        "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded lattice scene)",
        "config": {"workload": args.workload, "particles": n, "sand": sc.n_sand, "water": sc.n_water,
                   "boundary": sc.nb, "grid": list(sc.bparams.grid_size), "dt": dt,
                   "l2": ("working set ~250 B/particle > L2 (no flush needed)" if n >= 600_000 else
                          "working set < L2, not flushed (a profiling workload, not the benchmark)"),
                   "parallelism": f"replicas x{world}", "tuning": tuning},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic,
                     "traffic_source": traffic_source,
                     "algorithmic_bytes_per_particle": STAGE_BYTES[top]},
        "substep_roofline_frac": BYTES_PER_SUBSTEP * n / (ms / steps * 1e-3) / 1e9 / peak,
        "stage_ms": stage_ms,
        "pairs_per_substep": pairs,
        "pair_interactions_per_s": world * pairs * steps / (ms * 1e-3),
        "mean_neighbors": float(nbrs.mean()),
        "gpu_launches": launches,
        "device_error_flags": flags,
        "clocks": clk,
        "e2e": e2e,
        "bgeo_export": bgeo,
        "frame_adaptive": frame,
        "cpu_baseline": cpu,
        "batched": batched,
        "adjoint": adjoint,
        "calibration": calib,
        "long_run": longrun,
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line), flush=True)


def frame_timing(sim, n, frames=2):
    """The reference app's frame loop (sf_frame_adaptive, main.cpp:240-247):
    CFL substeps until 1/30 s has passed, each substep followed by the read of
    its substep count that the loop needs. Wall time over `frames` frames
    after one untimed frame, on the state the other measurements left."""
    interval = 1.0 / 30.0
    sim.frame_adaptive(interval)
    sim.synchronize()
    t0 = time.perf_counter()
    substeps = sum(sim.frame_adaptive(interval) for _ in range(frames))
    sim.synchronize()
    el = time.perf_counter() - t0
    return {"frames": frames, "substeps": substeps, "ms_per_substep": el / substeps * 1e3,
            "value": n * substeps / el, "unit": "particle-substeps/s",
            "path": "sf_frame_adaptive(1/30 s): sf_step per substep, N_sub read back after each"}


def bgeo_export_timing(sim, n):
    """sf_export_bgeo of the whole scene (the reference's per-frame export):
    wall time per call, GPU packing, device-to-host copy and file write
    included, into a RAM-backed folder where there is one."""
    import shutil
    import tempfile
    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    folder = tempfile.mkdtemp(prefix="sf_bgeo_", dir=base)
    try:
        sim.export_bgeo(folder, "warm")
        reps = 3
        t0 = time.perf_counter()
        for k in range(reps):
            sim.export_bgeo(folder, f"{k:04d}")
        el = (time.perf_counter() - t0) / reps
        size = os.path.getsize(os.path.join(folder, "0000.bgeo"))
    finally:
        shutil.rmtree(folder, ignore_errors=True)
    return {"particles": n, "file_bytes": size, "ms_per_export": el * 1e3, "file_gb_per_s": size / el / 1e9,
            "folder": "RAM-backed (/dev/shm)" if base else "temporary folder",
            "path": "sf_export_bgeo: GPU big-endian packing + D2H to pinned memory + file write"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain_large")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-calibration", action="store_true")
    ap.add_argument("--no-bgeo", action="store_true")
    ap.add_argument("--no-frame", action="store_true")
    ap.add_argument("--no-long-run", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--density-staging", default="auto", choices=["auto", "on", "off"],
                    help="density pass with or without shared-memory staging (default: the tuner's choice)")
    ap.add_argument("--adjoint-substeps", type=int, default=0,
                    help="only time the gradient run of the workload over this many substeps")
    ap.add_argument("--checkpoint-every", type=int, default=0,
                    help="checkpoint interval of --adjoint-substeps (default: every substep stored)")
    args = ap.parse_args()
    if args.adjoint_substeps > 0:
        adjoint_workload(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Shared helpers of the parity tests: fixture loading and error norms."""

import os

import numpy as np

from sph_seepage_flows_gb300.params import SfBoundaryParams, SfParams, SfSolverParams
from sph_seepage_flows_gb300.scenes import Scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def scene_from_golden(g, name="golden") -> Scene:
    p = SfParams.from_buffer_copy(g["params"].tobytes())
    b = SfBoundaryParams.from_buffer_copy(g["bparams"].tobytes())
    s = SfSolverParams.from_buffer_copy(g["sparams"].tobytes())
    return Scene(name=name, params=p, bparams=b, sparams=s, pos=g["in_pos"], vel=g["in_vel"], col=g["in_col"],
                 label=g["in_label"], mass=g["in_mass"], radius=g["in_radius"], cda0asat=g["in_cda0asat"],
                 amcamcp=g["in_amcamcp"], bpos=g["in_bpos"], blabel=g["in_blabel"])


def rel_err(a, b, scale=None, floor_frac=1e-3):
    """max over particles of |a - b| / max(scale, floor): scale defaults to
    |b| per particle (vector norm for vector fields), floor = floor_frac times
    the largest scale of the field."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    if d.ndim == 2:
        d = np.linalg.norm(d, axis=1)
    if scale is None:
        scale = np.linalg.norm(b, axis=1) if b.ndim == 2 else np.abs(b)
    scale = np.asarray(scale, np.float64)
    floor = floor_frac * (scale.max() if scale.size else 0.0) + 1e-30
    return float((d / np.maximum(scale, floor)).max()) if d.size else 0.0


def rel_err_q(a, b, scale=None, q=0.999, floor_frac=1e-3):
    """rel_err's per-particle errors at quantile q instead of the maximum."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    if d.ndim == 2:
        d = np.linalg.norm(d, axis=1)
    if scale is None:
        scale = np.linalg.norm(b, axis=1) if b.ndim == 2 else np.abs(b)
    scale = np.asarray(scale, np.float64)
    floor = floor_frac * (scale.max() if scale.size else 0.0) + 1e-30
    return float(np.quantile(d / np.maximum(scale, floor), q)) if d.size else 0.0


def exact_fraction(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    eq = (a == b)
    if eq.ndim == 2:
        eq = eq.all(1)
    return float(eq.mean()) if eq.size else 1.0


# Outputs of each stage of the substep that the stage-by-stage comparisons
# check, and the fields that pass through powf, the adhesion spline's fourth
# root or reordered sums (compared
# within tolerance; all others bit-for-bit).
STAGE_OUTPUTS = {
    "sort": ["id", "label", "pos", "vel", "col", "mass", "radius", "cda0asat", "amcamcp", "max_saturation"],
    "density": ["density", "pressure"],
    "avgflow": ["avg_flow", "voidage", "saturation"],
    "voidage_adhesion": ["voidage", "adhesion", "avg_adhesion", "col", "max_saturation"],
    "sand_momentum": ["acc", "avg_drag"],
    "water_momentum": ["acc"],
    "integrate": ["pos", "vel", "acc"],
}
TRANSCENDENTAL = {"pressure", "adhesion", "avg_adhesion", "acc", "avg_drag", "pos", "vel"}
CARRIED = ("pos", "vel", "acc", "density", "pressure", "voidage", "saturation", "avg_flow", "avg_drag", "adhesion",
           "avg_adhesion", "col", "max_saturation")


def compare_stages(sim, o32, time_arg, adaptive, tol, reps=1, stages=None, report=None):
    """Runs each stage of the substep on the GPU handle and on the FP32 oracle
    from identical inputs and checks every output: bit-for-bit, or within
    tol of the norm-relative error for the TRANSCENDENTAL fields (momentum
    accelerations against the oracle's per-particle sum of term magnitudes).
    After each stage the oracle takes the GPU's fields, so every stage sees
    the same inputs. report (a dict) collects (exact fraction, error)."""
    from sph_seepage_flows_gb300.params import STAGES
    for rep in range(reps):
        for st in (stages or STAGES):
            sim.stage(st, time_arg, adaptive=adaptive)
            o32.stage(st, time_arg, adaptive=adaptive)
            label = sim.field("label")
            for name in STAGE_OUTPUTS[st]:
                got = sim.field(name)
                ref = o32.field(name)
                keep = None
                if st == "sand_momentum":
                    keep = label == 1
                elif st == "water_momentum":
                    keep = label == 0
                if keep is not None:
                    got, ref = got[keep], ref[keep]
                frac = exact_fraction(got, ref)
                scale = None
                if name == "acc" and keep is not None:
                    # cancelling sums: measure against the sum of term magnitudes
                    scale = o32.field("acc_scale")[keep]
                err = rel_err(got, ref, scale)
                if report is not None:
                    report[(rep, st, name)] = (frac, err)
                if name in TRANSCENDENTAL:
                    assert err <= tol, (rep, st, name, err)
                else:
                    assert frac == 1.0, (rep, st, name, frac, err)
            for name in CARRIED:
                o32.set_field(name, sim.field(name))


def build_facade_program(tmp_path, name):
    """Compiles tests/cpp/<name>.cpp against the facade and libsf_gb300.so."""
    import subprocess
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / name)
    pkg = os.path.join(ROOT, "sph_seepage_flows_gb300")
    cmd = ["g++", "-std=c++17", "-O2", f'-DDB_PBR_PATH="{tmp_path}/"', "-I", os.path.join(ROOT, "include"),
           "-I", f"{cuda}/include",
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", exe, "-L", pkg, "-l:libsf_gb300.so",
           f"-Wl,-rpath,{pkg}", "-L", f"{cuda}/lib64", "-lcudart"]
    subprocess.run(cmd, check=True)
    return exe


def facade_scene(init_pos):
    """The scene the facade programs (tests/cpp/facade_scene.hpp) build, with
    their (seeded) initial positions."""
    from sph_seepage_flows_gb300 import scenes
    from sph_seepage_flows_gb300.params import SF_LABEL_SAND, SF_LABEL_WATER
    ns, nw = 8 * 6 * 8, 7 * 10 * 8
    sc = scenes.block_scene("facade", (0.4, 0.4, 0.4), (8, 6, 8), (7, 10, 8), 0.02, 0, jitter_frac=0.0,
                            sand_origin=(0.22, 0.02, 0.08), water_origin=(0.06, 0.02, 0.08))
    assert sc.n == ns + nw
    sc.pos = init_pos.astype(np.float32)
    sc.col = sc.col.copy()
    sc.col[sc.label == SF_LABEL_WATER] = np.array([0.5, 0.8, 1.0], np.float32)
    sc.cda0asat = np.zeros((sc.n, 3), np.float32)
    sc.cda0asat[sc.label == SF_LABEL_SAND] = [0.5, 0.0, 0.8]
    return sc

"""Writes the golden fixtures under tests/golden/ from the reference harness:
the sph_seepage_flows kernels compiled in place as host code
(oracle/ref_harness.cpp, built by oracle/build_ref.sh where the reference
sources are mounted). Run from the repository root:

    python tests/golden/make_golden.py

Fixtures (float32 / int32 arrays, cell-sorted order as the reference getters):
  tiny_multi_wcsph.npz  tiny scene, MULTI_SF + WCSPH: inputs, state after 1
                        and after 10 adaptive substeps (UpdateSystem(1/30))
  tiny_sf_sph.npz       same scene with SF + plain SPH: state after 1 substep
  tiny_plate.npz        tiny scene on a shape-boundary plate (label 1 boundary
                        particles): inputs, state after 1 substep
  emitters.npz          world-boundary shell and emitter sample points
  shapes.npz            the shape-volume builders on a seeded stand-in shape
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sph_seepage_flows_gb300 import scenes  # noqa: E402
from sph_seepage_flows_gb300.params import FIELDS, SF_SOLVER_SPH, SF_TYPE_SF  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
FIELD_NAMES = [k for k in FIELDS if k not in ("key", "neighbors")]


def cast(name, a):
    return a.astype(np.int32) if FIELDS.get(name, (0, 0, np.float32))[2] == np.int32 else a.astype(np.float32)


def inputs(sc):
    return {"in_" + k: getattr(sc, k) for k in ("pos", "vel", "col", "label", "mass", "radius", "cda0asat",
                                                "amcamcp", "bpos", "blabel")}


def snapshot(r, prefix, names=FIELD_NAMES):
    d = {f"{prefix}_{k}": cast(k, r.field(k)) for k in names}
    d[f"{prefix}_cell_start"] = r.cell_table(0).astype(np.int32)
    d[f"{prefix}_n_sub"] = np.int32(r.num_substeps)
    return d


def params_arrays(sc):
    return {"params": np.frombuffer(bytes(sc.params), dtype=np.uint8).copy(),
            "bparams": np.frombuffer(bytes(sc.bparams), dtype=np.uint8).copy(),
            "sparams": np.frombuffer(bytes(sc.sparams), dtype=np.uint8).copy()}


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference harness unavailable: the reference sources are not mounted")
    T = 1.0 / 30.0
    sc = scenes.tiny()
    r = oracle.RefHarness(sc)
    d = {**inputs(sc), **params_arrays(sc)}
    d["bcell_start"] = r.cell_table(1).astype(np.int32)
    d["bvolume"] = r.field("bvolume").astype(np.float32)
    d["bpos_sorted"] = r.field("bpos").astype(np.float32)
    r.substeps(T, True, 1)
    d.update(snapshot(r, "s1"))
    r.substeps(T, True, 9)
    d.update(snapshot(r, "s10", ["id", "label", "pos", "vel", "acc", "density", "pressure", "voidage",
                                 "saturation", "max_saturation", "col"]))
    np.savez_compressed(os.path.join(OUT, "tiny_multi_wcsph.npz"), **d)

    sc2 = scenes.tiny()
    sc2.params.sf_type = SF_TYPE_SF
    sc2.params.solver_type = SF_SOLVER_SPH
    r2 = oracle.RefHarness(sc2)
    d2 = {**inputs(sc2), **params_arrays(sc2)}
    r2.substeps(T, True, 1)
    d2.update(snapshot(r2, "s1"))
    np.savez_compressed(os.path.join(OUT, "tiny_sf_sph.npz"), **d2)

    lo, hi = (0.0, 0.0, 0.0), (0.4, 0.4, 0.4)
    wb, wl = oracle.ref_world_boundary(lo, hi, 0.01)
    wb2, _ = oracle.ref_world_boundary((0.0, 0.0, 0.0), (4.0, 0.6, 1.0), 0.005)
    em = {"world_boundary_small": wb, "world_boundary_small_label": wl,
          "world_boundary_large_count": np.int64(wb2.shape[0]),
          "world_boundary_large_sum": wb2.astype(np.float64).sum(0)}
    for kind, name, a, b in ((0, "square", 0.05, 0.0), (1, "circle", 0.17, 0.0), (2, "rectangle", 0.22, 0.18)):
        em["emit_" + name] = oracle.ref_emitter_points((0.9, 0.9, 1.25), (0.0, 0.0, -5.0), kind, 0.01, a, b)
    np.savez_compressed(os.path.join(OUT, "emitters.npz"), **em)
    shape_goldens()
    plate_golden()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)), "bytes")


def plate_golden():
    """Shape boundary particles in a substep: tiny scene on a label-1 plate."""
    sc = scenes.tiny_with_plate()
    r = oracle.RefHarness(sc)
    d = {**inputs(sc), **params_arrays(sc)}
    r.substeps(1.0 / 30.0, True, 1)
    d.update(snapshot(r, "s1"))
    np.savez_compressed(os.path.join(OUT, "tiny_plate.npz"), **d)


def shape_goldens():
    """The reference's shape-volume builders (the app's bunny/dam import path)
    on a seeded stand-in shape: 300 points in a ball with radii 4-6 mm."""
    import oracle
    rng = np.random.default_rng(2024)
    d = rng.normal(size=(300, 3))
    d *= (0.1 * rng.random(300) ** (1 / 3) / np.linalg.norm(d, axis=1))[:, None]
    shape = np.empty((300, 4), np.float32)
    shape[:, :3] = d + np.array([0.5, 0.3, 0.5])
    shape[:, 3] = 0.004 + 0.002 * rng.random(300)
    g = {"shape": shape}
    args = dict(color=(0.88, 0.79, 0.62), density=2650.0, cda0asat=(0.5, 0.6, 0.8), amcamcp=(0.7, 0.3))
    for tag, off, twice in (("plain", False, False), ("offset", True, False), ("offset_twice", True, True)):
        out = oracle.ref_shape_multi_volume(shape, offset_y=off, lowest_y=0.02, twice=twice, **args)
        for k, v in out.items():
            g[f"{tag}_{k}"] = v
    g["bshape_pos"], g["bshape_label"] = oracle.ref_boundary_shape_volume(shape)
    np.savez_compressed(os.path.join(OUT, "shapes.npz"), **g)


if __name__ == "__main__":
    main()

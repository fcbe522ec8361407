"""Writes tests/golden/refgpu_<scene>.npz: the state of the reference's own
CUDA library (seepage_flows_cuda built with its -use_fast_math flags by
oracle/build_ref_cuda.sh, driven through its public classes by
oracle/ref_gpu_driver.cu) after one UpdateSystem(1/30 s) call from each golden
scene's initial state. These are the device-arithmetic fixtures: they carry
the reference GPU path's results to places where its library is not built.

Needs a GPU and the staged reference sources (baseline/_ref/seepage_flows_cuda):

    python tests/golden/make_golden_refgpu.py [output folder (default: tests/golden)]

Each file holds, in the reference's current (sorted) order: id (creation
index), key (cell key of the step's sort), the fields after the step
(float32, as the device holds them), the particle and boundary cell tables,
the boundary positions, keys and Akinci volumes, and n_sub.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from helpers import load_golden, scene_from_golden  # noqa: E402

FIXTURES = ("tiny_multi_wcsph.npz", "tiny_sf_sph.npz", "tiny_plate.npz")
FIELDS = ("pos", "vel", "acc", "col", "density", "pressure", "voidage", "saturation", "max_saturation", "avg_flow",
          "avg_drag", "adhesion", "avg_adhesion")
T_FRAME = 1.0 / 30.0


def capture(scene):
    r = oracle.RefGpu(scene)
    r.update(T_FRAME)
    out = {"n_sub": np.int64(r.num_substeps), "id": r.field("id").astype(np.int32),
           "key": r.field("key").astype(np.int64), "cell_start": r.cell_table(0), "bcell_start": r.cell_table(1),
           "bkey": r.boundary_keys(), "bpos": r.field("bpos").astype(np.float32),
           "bvolume": r.field("bvolume").astype(np.float32)}
    for f in FIELDS:
        out[f] = r.field(f).astype(np.float32)
    return out


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(out_dir, exist_ok=True)
    if oracle.build_ref_gpu() is None:
        raise SystemExit("the reference CUDA library is not built (stage it with oracle/build_ref_cuda.sh)")
    for fx in FIXTURES:
        out = capture(scene_from_golden(load_golden(fx)))
        name = os.path.join(out_dir, "refgpu_" + fx)
        np.savez_compressed(name, **out)
        print("wrote", name, "n_sub", int(out["n_sub"]))


if __name__ == "__main__":
    main()

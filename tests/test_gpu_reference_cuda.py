"""The CUDA substep against the reference's own CUDA library on the GPU.

The reference's library (seepage_flows_cuda, built for sm_103a with its own
-use_fast_math flags by oracle/build_ref_cuda.sh and driven through its
public classes, oracle/ref_gpu_driver.cu) differs from the FP32 restatement
the other parity tests pin to in one way that matters for integer results:
its cell hash divides the position by the cell size with approximate
division (helper_thrust.cuh:58-60 under -use_fast_math). A particle lying
on a cell face (within a few float ulps of it) can therefore land in the
cell below. So:

* cell keys must agree for every particle and boundary particle, except
  particles whose quotient (p - lowest) / h lies within 4 ulps of an
  integer; every cell table must be the counting table of its own keys;
  where no key differs, the sorted ids and both tables are identical;
* after one substep, every field's error against the FP64 oracle (by
  particle id; worst particle and 99.9th percentile) is at most 4x the
  reference GPU path's own error against FP64, plus 1e-6.

The fixtures tests/golden/refgpu_*.npz (tests/golden/make_golden_refgpu.py)
carry the reference GPU path's results for the golden scenes; where the
reference library is built (the staged sources travel with the working tree)
the 40k and 1M configurations are compared live as well.
"""

import numpy as np
import pytest

from helpers import load_golden, rel_err, rel_err_q, scene_from_golden
from sph_seepage_flows_gb300 import scenes

pytestmark = pytest.mark.gpu

T_FRAME = 1.0 / 30.0
FIELDS = ("pos", "vel", "acc", "col", "density", "pressure", "voidage", "saturation", "max_saturation", "avg_flow",
          "avg_drag", "adhesion", "avg_adhesion")
FIXTURES = ("tiny_multi_wcsph.npz", "tiny_sf_sph.npz", "tiny_plate.npz")


def quotient_axes(bparams, pos):
    """(p - lowest) / h per axis in float32, as the IEEE cell hash forms it."""
    lp = np.asarray(bparams.lowest_point[:], np.float32)
    h = np.float32(bparams.kernel_radius)
    return (np.asarray(pos, np.float32) - lp) / h


def on_cell_face(bparams, pos, ulps=4):
    """Particles whose per-axis quotient lies within `ulps` float ulps of an
    integer on some axis (where approximate division can change the cell)."""
    q = quotient_axes(bparams, pos)
    near = np.abs(q - np.round(q)) <= ulps * np.spacing(np.abs(q).astype(np.float32))
    return near.any(axis=1)


def counting_table(keys, cells):
    return np.searchsorted(np.sort(keys), np.arange(cells + 1), side="left").astype(np.int64)


def check_keys(sc, ours_key_by_id, ref_key_by_id, pos_by_id, label):
    diff = ours_key_by_id != ref_key_by_id
    face = on_cell_face(sc.bparams, pos_by_id)
    unexplained = np.flatnonzero(diff & ~face)
    assert unexplained.size == 0, (label, unexplained[:10], int(diff.sum()))
    return int(diff.sum())


def error_report(ours, ref, o64, acc_scale):
    """{field: (ours-vs-FP64, ref-vs-FP64, ours-vs-ref)} as (max, 99.9%)."""
    rep = {}
    for f in FIELDS:
        scale = acc_scale if f == "acc" else None
        a, r, c = ours[f].astype(np.float64), ref[f].astype(np.float64), o64[f]
        rep[f] = ((rel_err(a, c, scale), rel_err_q(a, c, scale)), (rel_err(r, c, scale), rel_err_q(r, c, scale)),
                  (rel_err(a, r, scale), rel_err_q(a, r, scale)))
    return rep


def assert_as_accurate(rep, label):
    print(f"\n{label}: field  ours-vs-FP64 (max, 99.9%)  refGPU-vs-FP64  ours-vs-refGPU")
    for f, (o, r, c) in rep.items():
        print(f"  {f:15s} {o[0]:.2e} {o[1]:.2e}   {r[0]:.2e} {r[1]:.2e}   {c[0]:.2e} {c[1]:.2e}")
    for f, (o, r, _) in rep.items():
        assert o[1] <= 4.0 * r[1] + 1e-6, (label, f, "99.9%", o[1], r[1])
        assert o[0] <= 4.0 * r[0] + 1e-6, (label, f, "max", o[0], r[0])


def by_id(ids, a):
    out = np.empty_like(a)
    out[np.asarray(ids, np.int64)] = a
    return out


def ours_after_step(sc, steps=1):
    from sph_seepage_flows_gb300.capi import Simulation
    sim = Simulation(sc)
    nsub = 0
    for _ in range(steps):
        nsub = sim.step(T_FRAME)
    ids = sim.field("id")
    out = {f: by_id(ids, sim.field(f)) for f in FIELDS}
    out["key"] = by_id(ids, sim.field("key").astype(np.int64))
    out["id_sorted"] = ids
    out["cell_start"] = sim.cell_table(0)
    out["bcell_start"] = sim.cell_table(1)
    out["n_sub"] = nsub
    return out


def fp64_after_step(oracle_mod, sc, steps=1):
    o64 = oracle_mod.Oracle(sc, 64)
    o64.substeps(T_FRAME, True, steps)
    ids = o64.field("id").astype(np.int64)
    out = {f: by_id(ids, o64.field(f)) for f in FIELDS}
    out["acc_scale"] = by_id(ids, o64.field("acc_scale"))
    return out


def compare(oracle_mod, sc, ref, label):
    """ref: the reference GPU path's state after one step (sorted order)."""
    ours = ours_after_step(sc)
    assert ours["n_sub"] == int(ref["n_sub"]), label
    rid = np.asarray(ref["id"], np.int64)
    g = [int(v) for v in sc.bparams.grid_size]
    cells = g[0] * g[1] * g[2]
    # particle keys (of the step's sort: the initial positions)
    nflip = check_keys(sc, ours["key"], by_id(rid, np.asarray(ref["key"], np.int64)), sc.pos, label)
    assert np.array_equal(np.asarray(ref["cell_start"], np.int64), counting_table(np.asarray(ref["key"]), cells))
    assert np.array_equal(ours["cell_start"], counting_table(ours["key"], cells))
    if nflip == 0:
        assert np.array_equal(ours["id_sorted"].astype(np.int64), rid), label
        assert np.array_equal(ours["cell_start"], np.asarray(ref["cell_start"], np.int64)), label
    # boundary keys: the reference's boundary order against the IEEE hash of the same positions
    bpos = np.asarray(ref["bpos"], np.float32)
    q = np.clip(quotient_axes(sc.bparams, bpos).astype(np.int64), 0, np.array(g) - 1)
    ieee = (q[:, 0] * g[1] + q[:, 1]) * g[2] + q[:, 2]
    bdiff = ieee != np.asarray(ref["bkey"], np.int64)
    assert not (bdiff & ~on_cell_face(sc.bparams, bpos)).any(), label
    assert np.array_equal(np.asarray(ref["bcell_start"], np.int64), counting_table(np.asarray(ref["bkey"]), cells))
    assert np.array_equal(ours["bcell_start"], counting_table(ieee, cells))
    o64 = fp64_after_step(oracle_mod, sc)
    refd = {f: by_id(rid, np.asarray(ref[f])) for f in FIELDS}
    rep = error_report(ours, refd, o64, o64["acc_scale"])
    print(f"{label}: particle keys differing at cell faces {nflip}, boundary {int(bdiff.sum())} of {sc.nb}")
    assert_as_accurate(rep, label)


@pytest.mark.parametrize("fixture", FIXTURES)
def test_one_substep_against_reference_gpu_fixture(cuda_lib, oracle_mod, fixture):
    sc = scene_from_golden(load_golden(fixture))
    ref = load_golden("refgpu_" + fixture)
    compare(oracle_mod, sc, ref, fixture)


@pytest.fixture(scope="module")
def ref_gpu(oracle_mod):
    if oracle_mod.build_ref_gpu() is None:
        pytest.skip("the reference CUDA library is not staged here (oracle/build_ref_cuda.sh)")
    return oracle_mod


def ref_state(oracle_mod, sc):
    r = oracle_mod.RefGpu(sc)
    r.update(T_FRAME)
    out = {f: r.field(f).astype(np.float32) for f in FIELDS}
    out.update(n_sub=r.num_substeps, id=r.field("id").astype(np.int64), key=r.field("key").astype(np.int64),
               cell_start=r.cell_table(0), bcell_start=r.cell_table(1), bkey=r.boundary_keys(),
               bpos=r.field("bpos").astype(np.float32))
    return out


@pytest.mark.parametrize("which", ["plain_small", "plain_large"])
def test_one_substep_against_live_reference_gpu(cuda_lib, ref_gpu, which):
    sc = getattr(scenes, which)()
    compare(ref_gpu, sc, ref_state(ref_gpu, sc), which)

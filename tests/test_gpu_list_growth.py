"""Neighbour-list growth (sf_get_list_capacity). A density pass that finds a
particle's list more than 7/8 full records the particle's neighbour count;
the host reads that record after the call and re-allocates the lists (a
particle whose list overflowed meanwhile walks the stencil). Lists and
stencil walks visit the same neighbours in the same order, so a handle whose
lists grow computes the same states, bit for bit, as one created with lists
large enough from the start."""

import numpy as np
import pytest

from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import reference_dt

pytestmark = pytest.mark.gpu

FIELDS = ["pos", "vel", "acc", "density", "pressure", "voidage", "saturation", "avg_flow", "col"]


def compressed_positions(sc, factor=0.7):
    """The sand block compressed toward its centre: about 0.7^-3 = 2.9 times
    the lattice's ~30 neighbours, above the 64 list entries sized for the
    uncompressed scene and below the 256 the lists can grow to."""
    pos = sc.pos.copy()
    sand = sc.label == 1
    c = pos[sand].mean(0)
    pos[sand] = (c + factor * (pos[sand] - c)).astype(np.float32)
    return pos


def pair():
    """Handle A: created from the lattice (lists for ~30 neighbours), then
    given the compressed positions. Handle B: created from the compressed
    scene (lists sized for it)."""
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scenes.tiny(seed=12)
    squeezed = compressed_positions(sc)
    a = Simulation(sc)
    cap0, _ = a.list_capacity()
    a.set_field("pos", squeezed, order="id")
    sc_b = scenes.tiny(seed=12)
    sc_b.pos = squeezed
    b = Simulation(sc_b)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    return a, b, cap0, dt


def fields(sim):
    return {f: sim.field(f, order="id") for f in FIELDS}


def test_lists_grow_at_the_next_call(cuda_lib):
    a, b, cap0, dt = pair()
    cap_b, growths_b = b.list_capacity()
    assert cap0 == 64 and growths_b == 0
    a.substeps_fixed(dt, 1)
    b.substeps_fixed(dt, 1)
    need = int(b.field("neighbors").max())
    assert 64 < need <= 256 and cap_b >= need
    a.synchronize()
    assert a.list_capacity() == (64, 0)   # the record is read by the next stepping call
    a.substeps_fixed(dt, 3)
    b.substeps_fixed(dt, 3)
    cap_a, growths_a = a.list_capacity()
    assert growths_a == 1 and cap_a % 32 == 0 and cap_a >= need
    fa, fb = fields(a), fields(b)
    for f in FIELDS:
        assert np.array_equal(fa[f], fb[f], equal_nan=True), f
    assert a.check_error() == b.check_error()
    a.close()
    b.close()


def test_lists_grow_within_a_long_call(cuda_lib):
    """A call of more than 64 substeps waits, after each block of 64, for
    the block before it, and grows the lists there: the capacity has grown
    when the call returns."""
    a, b, cap0, dt = pair()
    assert cap0 == 64
    a.substeps_fixed(dt, 600)
    cap_a, growths_a = a.list_capacity()
    assert growths_a >= 1 and cap_a > 64
    b.substeps_fixed(dt, 600)
    fa, fb = fields(a), fields(b)
    for f in FIELDS:
        assert np.array_equal(fa[f], fb[f], equal_nan=True), f
    a.close()
    b.close()

"""sf_cell_sort_noalloc (static device scratch, no allocation) against the
sort stage of a handle on the same positions, through the C ABI.

Integer results, so the bar is bit-exactness: the permutation must equal the
ids of the handle's particles in sorted order and the cell-start table must
equal the handle's, on two calls in a row (the second call reuses the
scratch the first one left behind).
"""

import ctypes

import numpy as np
import pytest

from sph_seepage_flows_gb300 import scenes

pytestmark = pytest.mark.gpu


def _call(lib, bparams, pos, n, perm, cs):
    return lib.sf_cell_sort_noalloc(ctypes.byref(bparams), ctypes.c_void_p(pos), ctypes.c_int64(n),
                                    ctypes.c_void_p(perm), ctypes.c_void_p(cs), None)


@pytest.mark.parametrize("name", ["tiny", "plain_small"])
def test_noalloc_sort_matches_sort_stage(cuda_lib, name):
    torch = pytest.importorskip("torch")
    from sph_seepage_flows_gb300.capi import Simulation
    sc = getattr(scenes, name)()
    sim = Simulation(sc)
    sim.stage("sort")
    ids = sim.field("id", order="sorted").astype(np.int64)
    table = sim.cell_table(0)
    sim.close()
    g = len(table) - 1
    pos = torch.tensor(np.ascontiguousarray(sc.pos), device="cuda")
    for call in range(2):
        perm = torch.full((sc.n,), -1, dtype=torch.int32, device="cuda")
        cs = torch.full((g + 1,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = _call(cuda_lib, sc.bparams, pos.data_ptr(), sc.n, perm.data_ptr(), cs.data_ptr())
        assert st == 0, cuda_lib.sf_last_error_string(None).decode()
        torch.cuda.synchronize()
        assert np.array_equal(perm.cpu().numpy().astype(np.int64), ids), f"call {call}"
        assert np.array_equal(cs.cpu().numpy().astype(np.int64), table), f"call {call}"


def test_noalloc_rejects_oversize(cuda_lib):
    torch = pytest.importorskip("torch")
    sc = scenes.tiny()
    max_n = 262144
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = _call(cuda_lib, sc.bparams, buf.data_ptr(), max_n + 1, buf.data_ptr(), buf.data_ptr())
    assert st == 1
    assert "SF_NOALLOC_MAX_PARTICLES" in cuda_lib.sf_last_error_string(None).decode()


def _grid_keys(bparams, pos):
    """Pos2GridHash in float32: per-axis truncation of (p - lowest) / h,
    clamped to the grid (the key of the sort stage)."""
    lp = np.asarray(bparams.lowest_point[:], np.float32)
    h = np.float32(bparams.kernel_radius)
    g = np.asarray(bparams.grid_size[:], np.int64)
    c = ((pos.astype(np.float32) - lp) / h).astype(np.int64)
    c = np.clip(c, 0, g - 1)
    return (c[:, 0] * g[1] + c[:, 1]) * g[2] + c[:, 2], int(g.prod())


def test_noalloc_at_max_size_matches_numpy_stable_sort(cuda_lib):
    """n = SF_NOALLOC_MAX_PARTICLES (the most sort tiles the static histogram
    scratch has to hold): the permutation equals numpy's stable argsort of
    the cell keys and the table its left search over cell indices."""
    torch = pytest.importorskip("torch")
    sc = scenes.plain_small()
    n = 262144
    rng = np.random.default_rng(3)
    # positions spread over the 1 m box, a few of them outside it (clamped cells)
    pos = rng.uniform(-0.02, 1.02, size=(n, 3)).astype(np.float32)
    keys, g = _grid_keys(sc.bparams, pos)
    want = np.argsort(keys, kind="stable")
    table = np.searchsorted(keys[want], np.arange(g + 1), side="left")
    dpos = torch.tensor(pos, device="cuda")
    for call in range(2):
        perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        cs = torch.full((g + 1,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = _call(cuda_lib, sc.bparams, dpos.data_ptr(), n, perm.data_ptr(), cs.data_ptr())
        assert st == 0, cuda_lib.sf_last_error_string(None).decode()
        assert np.array_equal(perm.cpu().numpy(), want), f"call {call}"
        assert np.array_equal(cs.cpu().numpy(), table), f"call {call}"


def test_noalloc_empty_input_gives_zero_table(cuda_lib):
    torch = pytest.importorskip("torch")
    sc = scenes.tiny()
    g = int(np.prod(np.asarray(sc.bparams.grid_size[:], np.int64)))
    cs = torch.full((g + 1,), -1, dtype=torch.int32, device="cuda")
    perm = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = _call(cuda_lib, sc.bparams, perm.data_ptr(), 0, perm.data_ptr(), cs.data_ptr())
    assert st == 0, cuda_lib.sf_last_error_string(None).decode()
    torch.cuda.synchronize()
    assert not cs.cpu().numpy().any()


def test_noalloc_reports_nonfinite_position(cuda_lib):
    """A NaN position (its key still lands in a valid cell) is reported as
    SF_ERR_DEVICE; the next call with finite positions succeeds, since the
    flag is cleared by every call."""
    torch = pytest.importorskip("torch")
    sc = scenes.tiny()
    g = int(np.prod(np.asarray(sc.bparams.grid_size[:], np.int64)))
    pos = np.ascontiguousarray(sc.pos).copy()
    pos[5, 1] = np.nan
    dpos = torch.tensor(pos, device="cuda")
    perm = torch.zeros(sc.n, dtype=torch.int32, device="cuda")
    cs = torch.zeros(g + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = _call(cuda_lib, sc.bparams, dpos.data_ptr(), sc.n, perm.data_ptr(), cs.data_ptr())
    assert st == 4, st
    assert "non-finite" in cuda_lib.sf_last_error_string(None).decode()
    dpos = torch.tensor(np.ascontiguousarray(sc.pos), device="cuda")
    st = _call(cuda_lib, sc.bparams, dpos.data_ptr(), sc.n, perm.data_ptr(), cs.data_ptr())
    assert st == 0, cuda_lib.sf_last_error_string(None).decode()


def test_noalloc_allocates_no_device_memory(cuda_lib):
    """After a warm-up call (module loaded, scratch address known), further
    calls leave the device's free memory and torch's allocator unchanged."""
    torch = pytest.importorskip("torch")
    sc = scenes.plain_small()
    g = int(np.prod(np.asarray(sc.bparams.grid_size[:], np.int64)))
    dpos = torch.tensor(np.ascontiguousarray(sc.pos), device="cuda")
    perm = torch.zeros(sc.n, dtype=torch.int32, device="cuda")
    cs = torch.zeros(g + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert _call(cuda_lib, sc.bparams, dpos.data_ptr(), sc.n, perm.data_ptr(), cs.data_ptr()) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for _ in range(3):
        assert _call(cuda_lib, sc.bparams, dpos.data_ptr(), sc.n, perm.data_ptr(), cs.data_ptr()) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_allocated() == alloc0

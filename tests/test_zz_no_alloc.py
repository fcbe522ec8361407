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

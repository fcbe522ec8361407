"""The GPU .bgeo export (sf_export_bgeo, sf_export_bgeo_device) against the
oracle's writer and partio's: the files are byte-identical to the oracle's
for the same particle arrays (the handle's current, cell-sorted order) and to
the bytes partio's own writer produced for the committed point set
(tests/golden/partio_export.npz), they read back through sf_read_bgeo, and
the 1M-particle scene's export parses to exactly its fields."""

import numpy as np
import pytest

from oracle import bgeo
from sph_seepage_flows_gb300 import scenes
from sph_seepage_flows_gb300.params import reference_dt

pytestmark = pytest.mark.gpu


def sorted_fields(sim):
    return (sim.field("pos"), sim.field("col"), sim.field("radius"), sim.field("label"))


def test_handle_export_is_byte_identical(cuda_lib, tmp_path):
    from sph_seepage_flows_gb300.capi import Simulation, read_bgeo
    sc = scenes.tiny(seed=4)
    sim = Simulation(sc)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    sim.substeps_fixed(dt, 5)
    folder = tmp_path / "frames" / "run"   # created by the export
    sim.export_bgeo(str(folder), "0001")
    data = (folder / "0001.bgeo").read_bytes()
    pos, col, rad, lab = sorted_fields(sim)
    assert data == bgeo.write_bytes(pos, col, rad, lab)
    back = read_bgeo(str(folder / "0001.bgeo"))
    assert np.array_equal(back[:, :3], pos) and np.array_equal(back[:, 3], rad)
    sim.close()


def test_device_array_export_is_byte_identical(cuda_lib, tmp_path):
    import torch
    from sph_seepage_flows_gb300.capi import export_bgeo_device
    for n in (0, 1, 255, 256, 1000):
        rng = np.random.default_rng(n)
        pos = rng.normal(size=(n, 3)).astype(np.float32)
        col = rng.random((n, 3)).astype(np.float32)
        rad = (rng.random(n) * 0.01).astype(np.float32)
        lab = rng.integers(0, 2, n).astype(np.int64)
        t = [torch.from_numpy(a).cuda() for a in (pos, col, rad, lab)]
        stream = torch.cuda.current_stream().cuda_stream
        export_bgeo_device(str(tmp_path), f"d{n}", *[x.data_ptr() if n else 0 for x in t], n, stream)
        assert (tmp_path / f"d{n}.bgeo").read_bytes() == bgeo.write_bytes(pos, col, rad, lab), n


def test_device_array_export_equals_partio_bytes(cuda_lib, tmp_path):
    import torch

    from helpers import load_golden
    from sph_seepage_flows_gb300.capi import export_bgeo_device
    g = load_golden("partio_export.npz")
    t = [torch.from_numpy(np.ascontiguousarray(g[k])).cuda() for k in ("pos", "col", "radius", "label")]
    stream = torch.cuda.current_stream().cuda_stream
    export_bgeo_device(str(tmp_path), "partio", *[x.data_ptr() for x in t], len(g["radius"]), stream)
    assert (tmp_path / "partio.bgeo").read_bytes() == g["bgeo"].tobytes()


def test_large_scene_export_parses_to_its_fields(cuda_lib, tmp_path):
    from sph_seepage_flows_gb300.capi import Simulation
    sc = scenes.plain_large()
    sim = Simulation(sc)
    dt = reference_dt(sc.params, sc.bparams, sc.sparams)[1]
    sim.substeps_fixed(dt, 2)
    sim.export_bgeo(str(tmp_path), "big")
    a = bgeo.read((tmp_path / "big.bgeo").read_bytes())
    pos, col, rad, lab = sorted_fields(sim)
    assert np.array_equal(a["position"], pos) and np.array_equal(a["Cd"], col)
    assert np.array_equal(a["pscale"][:, 0], rad) and np.array_equal(a["label"][:, 0], lab)
    sim.close()


def test_batched_handle_exports_each_scene(cuda_lib, tmp_path):
    """Each scene of a batched handle exports its own particles (its slot
    range of the scene-offset layout), equal to a single-scene handle's file."""
    from sph_seepage_flows_gb300.capi import Simulation
    scs = [scenes.tiny(seed=s) for s in (7, 8, 9)]
    scs[1] = scenes.tiny(seed=8, sand=(6, 6, 6), water=(5, 7, 6))   # a different size
    dt = reference_dt(scs[0].params, scs[0].bparams, scs[0].sparams)[1]
    sim = Simulation(scs)
    sim.substeps_fixed(dt, 3)
    for k, sc in enumerate(scs):
        sim.export_bgeo(str(tmp_path), f"scene{k}", scene=k)
        one = Simulation(sc)
        one.substeps_fixed(dt, 3)
        one.export_bgeo(str(tmp_path), f"single{k}")
        assert (tmp_path / f"scene{k}.bgeo").read_bytes() == (tmp_path / f"single{k}.bgeo").read_bytes(), k
        one.close()
    sim.close()

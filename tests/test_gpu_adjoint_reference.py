"""The GPU adjoint against a reference gradient: the exact pathwise
directional derivatives of the FP64 forward-mode oracle (precision 65, one
dual-number tangent carried through the restatement of the reference
kernels).

Cases: the smooth probes of test_gpu_adjoint.py, and the DEM-contact probes
(every sand lattice pair overlapping, sliding contacts at the friction cap),
where central differences only converge at the finest step because of the
friction-cap kinks, so the forward-mode oracle is the reference.

Tolerance: 1e-3 relative (the gradient accuracy target).

Not compared: scenes whose trajectories cross the model's value
discontinuities densely (the 20k-particle column: lattice pairs straddle the
liquid-bridge onset H = 0, sand voidage is near 0 where the drag goes as
1 / voidage, the damping factor switches sign). There the FP32 trajectory of
the GPU and the FP64 trajectory of the oracle take different branches within
a few substeps and their pathwise derivatives differ; central differences do
not converge either (test_adjoint_fd_cpu.py documents the probes where they do).
"""

import numpy as np
import pytest

from fd_oracle import (CONTACT_CASES, DT, PROBE_CASES, contact_scene, jvp, probe_direction, probe_scene,
                       probe_target)

pytestmark = pytest.mark.gpu

TOL = 1e-3
PARAMS = ("tan", "cap", "perm")
CASES = [("probe",) + c for c in PROBE_CASES] + [("contact",) + c for c in CONTACT_CASES]


def make(case):
    if case[0] == "probe":
        return probe_scene(case[1], case[3]), case[2]
    return contact_scene(case[1], case[3], case[4]), case[2]


@pytest.fixture(scope="module")
def runs(cuda_lib):
    """Gradients with the automatic lane count (8 threads per particle on these
    small scenes) and with one (the path of large scenes)."""
    from sph_seepage_flows_gb300.capi import Simulation
    out = {}
    for case in CASES:
        for lanes in (0, 1):
            sc, n_sub = make(case)
            sim = Simulation(sc)
            sim.set_lanes(lanes)
            out[case, lanes] = (sc, n_sub, sim.adjoint(DT, n_sub, probe_target(sc)))
            sim.close()
    return out


@pytest.mark.parametrize("lanes", [0, 1])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}")
@pytest.mark.parametrize("which", ["pos", "vel"] + list(PARAMS))
def test_adjoint_against_forward_mode(runs, oracle_mod, case, which, lanes):
    sc, n_sub, res = runs[case, lanes]
    target = probe_target(sc)
    if which in ("pos", "vel"):
        u = probe_direction(sc, case[1])
        ref = jvp(oracle_mod, sc, DT, n_sub, target, which, u)
        ad = float(np.sum(res["grad_pos0" if which == "pos" else "grad_vel0"].astype(np.float64) * u))
    else:
        ref = jvp(oracle_mod, sc, DT, n_sub, target, which)
        ad = float(res["grad_params"][0, PARAMS.index(which)])
    if ref == 0.0:  # no liquid bridges in the contact probes: the capillary scale has no effect
        assert ad == 0.0
        return
    assert abs(ad - ref) <= TOL * abs(ref), (ad, ref)

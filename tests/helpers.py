"""Shared helpers of the parity tests: fixture loading and error norms."""

import os

import numpy as np

from sph_seepage_flows_gb300.params import SfBoundaryParams, SfParams, SfSolverParams
from sph_seepage_flows_gb300.scenes import Scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


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


def exact_fraction(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    eq = (a == b)
    if eq.ndim == 2:
        eq = eq.all(1)
    return float(eq.mean()) if eq.size else 1.0

"""Parameter structs of the C ABI (include/sf_capi.h) as ctypes structures.

The fields mirror the reference's global parameter structs:
``CudaSeepageflowParams`` (seepage_flows_cuda/include/kiri_pbs_cuda/data/cuda_seepageflow_params.h:25-69),
``CudaBoundaryParams`` (.../data/cuda_boundary_params.h:19-27) and the
``CudaWCSphSFSolver`` constructor arguments (.../solver/seepageflow/cuda_wcsph_sf_solver.cuh:22-32).
:func:`reference_params` reproduces the values the reference app sets in
``SetupParams`` (seepage_flows/src/seepageflow/main.cpp:40-83).
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

SF_SOLVER_SPH = 0
SF_SOLVER_WCSPH = 1
SF_TYPE_SF = 0
SF_TYPE_MULTI_SF = 1
SF_LABEL_WATER = 0
SF_LABEL_SAND = 1

# field ids (include/sf_capi.h)
FIELDS = {
    "pos": (0, 3, np.float32), "vel": (1, 3, np.float32), "acc": (2, 3, np.float32),
    "col": (3, 3, np.float32), "label": (4, 1, np.int32), "radius": (5, 1, np.float32),
    "mass": (6, 1, np.float32), "density": (7, 1, np.float32), "pressure": (8, 1, np.float32),
    "voidage": (9, 1, np.float32), "saturation": (10, 1, np.float32),
    "max_saturation": (11, 1, np.float32), "avg_flow": (12, 3, np.float32),
    "avg_drag": (13, 3, np.float32), "adhesion": (14, 3, np.float32),
    "avg_adhesion": (15, 3, np.float32), "cda0asat": (16, 3, np.float32),
    "amcamcp": (17, 2, np.float32), "id": (18, 1, np.int32), "key": (19, 1, np.int32),
    "neighbors": (20, 1, np.int32),
}
BFIELDS = {"bpos": (32, 3, np.float32), "blabel": (33, 1, np.int32), "bvolume": (34, 1, np.float32)}

STAGES = ["sort", "density", "avgflow", "voidage_adhesion", "sand_momentum", "water_momentum", "integrate"]
STAGE_ID = {name: i for i, name in enumerate(STAGES)}


class SfParams(ctypes.Structure):
    _fields_ = [
        ("sph_mass", ctypes.c_float), ("sph_density", ctypes.c_float),
        ("sph_particle_radius", ctypes.c_float), ("sph_kernel_radius", ctypes.c_float),
        ("sph_stiff", ctypes.c_float), ("sph_visc", ctypes.c_float),
        ("sph_nu", ctypes.c_float), ("sph_bnu", ctypes.c_float),
        ("dem_mass", ctypes.c_float), ("dem_density", ctypes.c_float),
        ("dem_particle_radius", ctypes.c_float), ("dem_kernel_radius", ctypes.c_float),
        ("dem_young", ctypes.c_float), ("dem_poisson", ctypes.c_float),
        ("dem_tan_friction_angle", ctypes.c_float), ("dem_damping", ctypes.c_float),
        ("sf_c0", ctypes.c_float), ("sf_csat", ctypes.c_float), ("sf_cmc", ctypes.c_float),
        ("sf_cmc_p", ctypes.c_float), ("sf_cd", ctypes.c_float),
        ("sf_a0", ctypes.c_float), ("sf_asat", ctypes.c_float), ("sf_amc", ctypes.c_float),
        ("sf_amc_p", ctypes.c_float),
        ("sf_dry_sand_color", ctypes.c_float * 3), ("sf_wet_sand_color", ctypes.c_float * 3),
        ("gravity", ctypes.c_float * 3), ("dt", ctypes.c_float),
        ("solver_type", ctypes.c_int32), ("sf_type", ctypes.c_int32),
    ]

    def to_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, ctypes.Array) else v
        return out

    @classmethod
    def from_dict(cls, d: dict) -> "SfParams":
        p = cls()
        for name, _ in cls._fields_:
            if name in d:
                v = d[name]
                if isinstance(getattr(p, name), ctypes.Array):
                    getattr(p, name)[:] = [float(x) for x in v]
                else:
                    setattr(p, name, v)
        return p


class SfBoundaryParams(ctypes.Structure):
    _fields_ = [
        ("kernel_radius", ctypes.c_float),
        ("lowest_point", ctypes.c_float * 3), ("highest_point", ctypes.c_float * 3),
        ("world_size", ctypes.c_float * 3), ("world_center", ctypes.c_float * 3),
        ("grid_size", ctypes.c_int32 * 3),
    ]

    def to_dict(self) -> dict:
        return {name: list(getattr(self, name)) if name != "kernel_radius" else self.kernel_radius
                for name, _ in self._fields_}

    @classmethod
    def from_dict(cls, d: dict) -> "SfBoundaryParams":
        b = cls()
        b.kernel_radius = float(d["kernel_radius"])
        for name in ("lowest_point", "highest_point", "world_size", "world_center"):
            getattr(b, name)[:] = [float(x) for x in d[name]]
        b.grid_size[:] = [int(x) for x in d["grid_size"]]
        return b


class SfSolverParams(ctypes.Structure):
    _fields_ = [("negative_scale", ctypes.c_float), ("time_step_limit_scale", ctypes.c_float),
                ("speed_of_sound", ctypes.c_float)]


class SfSceneInit(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("pos", ctypes.POINTER(ctypes.c_float)), ("vel", ctypes.POINTER(ctypes.c_float)),
        ("col", ctypes.POINTER(ctypes.c_float)), ("label", ctypes.POINTER(ctypes.c_int32)),
        ("mass", ctypes.POINTER(ctypes.c_float)), ("radius", ctypes.POINTER(ctypes.c_float)),
        ("cda0asat", ctypes.POINTER(ctypes.c_float)), ("amcamcp", ctypes.POINTER(ctypes.c_float)),
        ("nb", ctypes.c_int64),
        ("bpos", ctypes.POINTER(ctypes.c_float)), ("blabel", ctypes.POINTER(ctypes.c_int32)),
    ]


def f32(x) -> float:
    """Round a Python float to the nearest float32 value."""
    return float(np.float32(x))


def grid_size_of(lowest, highest, cell) -> list:
    """make_int3((highest - lowest) / cell) in float32 with truncation
    (cuda_neighbor_searcher.cu:27, helper_math.h:185)."""
    lo = np.asarray(lowest, dtype=np.float32)
    hi = np.asarray(highest, dtype=np.float32)
    q = (hi - lo) / np.float32(cell)
    return [int(v) for v in q.astype(np.float32)]


def reference_params(sph_radius: float = 0.01, dem_radius: float = 0.01, dem_density: float = 2650.0,
                     gravity_y: float = -9.81, sf_type: int = SF_TYPE_MULTI_SF,
                     solver_type: int = SF_SOLVER_WCSPH) -> SfParams:
    """The reference parameter set of main.cpp:40-83 in float32 arithmetic,
    with the sand radius/density and gravity of the benchmark configs."""
    p = SfParams()
    r = np.float32(sph_radius)
    p.sph_density = 1000.0
    p.sph_particle_radius = float(r)
    h = np.float32(4.0) * r
    p.sph_kernel_radius = float(h)
    diam = np.float32(2.0) * r
    p.sph_mass = float(np.float32(0.8) * diam * diam * diam * np.float32(1000.0))
    visc = np.float32(0.05)
    c = np.float32(100.0)
    p.sph_nu = float((visc + visc) * h * c)
    p.sph_bnu = float(np.float32(0.2) * h * c)
    p.sph_stiff = float(np.float32(0.001) * c * c * np.float32(1000.0) / np.float32(7.0))
    p.sph_visc = float(visc)
    rd = np.float32(dem_radius)
    p.dem_density = float(np.float32(dem_density))
    p.dem_particle_radius = float(rd)
    p.dem_mass = float(np.float32(dem_density) * (np.float32(4.0) / np.float32(3.0) * np.float32(3.1415926)
                                                  * np.float32(rd) ** np.float32(3)))
    p.dem_kernel_radius = 0.0
    p.dem_young = 1e5
    p.dem_poisson = 0.3
    p.dem_tan_friction_angle = 0.5
    p.dem_damping = 0.4
    p.sf_c0, p.sf_cd, p.sf_csat, p.sf_cmc, p.sf_cmc_p = 0.7, 0.5, 0.0, 1.0, 0.01
    p.sf_a0, p.sf_asat, p.sf_amc, p.sf_amc_p = 0.0, 0.8, 1.5, 0.5
    p.sf_dry_sand_color[:] = [0.88, 0.79552, 0.5984]
    p.sf_wet_sand_color[:] = [0.38, 0.29, 0.14]
    p.dt = float(np.float32(0.5) * rd / np.sqrt(np.float32(1e5) / np.float32(dem_density)).astype(np.float32))
    p.gravity[:] = [0.0, gravity_y, 0.0]
    p.solver_type = solver_type
    p.sf_type = sf_type
    return p


def boundary_params(lowest, highest, kernel_radius: float) -> SfBoundaryParams:
    """CUDA_BOUNDARY_PARAMS as main.cpp:94-101 fills them."""
    b = SfBoundaryParams()
    lo = np.asarray(lowest, dtype=np.float32)
    hi = np.asarray(highest, dtype=np.float32)
    b.kernel_radius = f32(kernel_radius)
    b.lowest_point[:] = [float(v) for v in lo]
    b.highest_point[:] = [float(v) for v in hi]
    b.world_size[:] = [float(v) for v in (hi - lo)]
    b.world_center[:] = [float(v) for v in (hi + lo) / np.float32(2.0)]
    b.grid_size[:] = grid_size_of(lo, hi, kernel_radius)
    return b


def solver_params(negative_scale: float = 0.0, time_step_limit_scale: float = 3.0,
                  speed_of_sound: float = 100.0) -> SfSolverParams:
    s = SfSolverParams()
    s.negative_scale = negative_scale
    s.time_step_limit_scale = time_step_limit_scale
    s.speed_of_sound = speed_of_sound
    return s


def reference_dt(p: SfParams, b: SfBoundaryParams, s: SfSolverParams, render_interval: float = 1.0 / 30.0):
    """Sub-step count and dt of the WCSPH CFL rule at rest (force limit not
    binding): (N_sub, dt) with dt = T / N_sub (cuda_wcsph_sf_solver.cu:35-58)."""
    by_speed = np.float32(0.4) * np.float32(b.kernel_radius) / np.float32(s.speed_of_sound)
    desired = min(np.float32(s.time_step_limit_scale) * by_speed, np.float32(p.dt))
    n_sub = int(np.float32(render_interval) / np.float32(desired))
    return n_sub, float(np.float32(render_interval) / np.float32(n_sub))


def tan_deg(deg: float) -> float:
    return math.tan(math.radians(deg))

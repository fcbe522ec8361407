"""ORACLE -- test infrastructure, not product code.

ctypes wrappers of the CPU oracle (oracle/sf_oracle.cpp -> oracle/libsforacle.so),
of the reference harness (oracle/ref_harness.cpp -> oracle/_ref/libsfref.so,
built only where the reference sources are mounted) and of the reference's
own CUDA library driven through its public classes (oracle/ref_gpu_driver.cu
-> baseline/_ref/libsfrefgpu.so, built by oracle/build_ref_cuda.sh from the
staged reference sources). Only tests/, __graft_entry__.smoke() and bench.py's
baseline legs use this package, and only as the checker of the CUDA path or
as the baseline it is timed against.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from sph_seepage_flows_gb300.params import BFIELDS, FIELDS, STAGE_ID, SfBoundaryParams, SfParams, SfSceneInit, \
    SfSolverParams

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libsforacle.so")
REF_SO = os.path.join(HERE, "_ref", "libsfref.so")
REF_GPU_SO = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "libsfrefgpu.so")


def build(force: bool = False) -> str:
    """Compile the oracle library (make -C oracle)."""
    if force or not os.path.exists(ORACLE_SO) or \
            os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "sf_oracle.cpp")):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", HERE, "libsforacle.so"], check=True)
    return ORACLE_SO


def build_ref() -> str | None:
    """Compile the reference harness when the reference sources are present."""
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True)
    return REF_SO if os.path.exists(REF_SO) else None


def build_ref_gpu() -> str | None:
    """Stage (where the reference sources are mounted) and compile (where the
    staged copy exists) the reference's CUDA library with its driver."""
    subprocess.run(["sh", os.path.join(HERE, "build_ref_cuda.sh")], check=True)
    return REF_GPU_SO if os.path.exists(REF_GPU_SO) else None


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if a is not None else None


class SceneInit:
    """Keeps the numpy buffers of an sf_scene_init alive."""

    def __init__(self, scene):
        self.arrays = {}
        for name in ("pos", "vel", "col", "mass", "radius", "cda0asat", "amcamcp", "bpos"):
            self.arrays[name] = np.ascontiguousarray(getattr(scene, name), dtype=np.float32)
        for name in ("label", "blabel"):
            self.arrays[name] = np.ascontiguousarray(getattr(scene, name), dtype=np.int32)
        a = self.arrays
        self.init = SfSceneInit(n=scene.n, pos=_fptr(a["pos"]), vel=_fptr(a["vel"]), col=_fptr(a["col"]),
                                label=_iptr(a["label"]), mass=_fptr(a["mass"]), radius=_fptr(a["radius"]),
                                cda0asat=_fptr(a["cda0asat"]), amcamcp=_fptr(a["amcamcp"]), nb=scene.nb,
                                bpos=_fptr(a["bpos"]), blabel=_iptr(a["blabel"]))


def _field_meta(name):
    if name in FIELDS:
        return FIELDS[name]
    if name in BFIELDS:
        return BFIELDS[name]
    if name == "acc_scale":
        return (100, 1, np.float64)
    if name == "pressure_scale":
        return (101, 1, np.float64)
    raise KeyError(name)


class _Base:
    _lib = None
    _prefix = ""

    def field(self, name: str) -> np.ndarray:
        fid, width, _ = _field_meta(name)
        count = self.nb if fid >= 32 and fid < 100 else self.n
        out = np.zeros(count * width, dtype=np.float64)
        rc = getattr(self._lib, self._prefix + "get_field")(self.h, fid, out.ctypes.data_as(
            ctypes.POINTER(ctypes.c_double)), ctypes.c_int64(count))
        if rc != 0:
            raise RuntimeError(f"get_field({name}) failed: {rc}")
        return out.reshape(count, width) if width > 1 else out

    def fields(self, names=None) -> dict:
        names = names or list(FIELDS.keys())
        return {k: self.field(k) for k in names}

    def cell_table(self, which: int = 0) -> np.ndarray:
        g = np.asarray(self.bparams.grid_size[:], dtype=np.int64)
        count = int(g.prod()) + 1
        out = np.zeros(count, dtype=np.int64)
        rc = getattr(self._lib, self._prefix + "get_cell_table")(self.h, which, out.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int64)), ctypes.c_int64(count))
        if rc != 0:
            raise RuntimeError("get_cell_table failed")
        return out

    def __del__(self):
        try:
            if getattr(self, "h", None):
                getattr(self._lib, self._prefix + "destroy")(self.h)
                self.h = None
        except Exception:
            pass


def _load_oracle():
    build()
    lib = ctypes.CDLL(ORACLE_SO)
    lib.sfo_create.restype = ctypes.c_void_p
    lib.sfo_create.argtypes = [ctypes.c_int, ctypes.POINTER(SfParams), ctypes.POINTER(SfBoundaryParams),
                               ctypes.POINTER(SfSolverParams), ctypes.POINTER(SfSceneInit), ctypes.c_int]
    lib.sfo_destroy.argtypes = [ctypes.c_void_p]
    lib.sfo_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
    lib.sfo_set_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
    lib.sfo_get_cell_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                       ctypes.c_int64]
    lib.sfo_run_stage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.sfo_substeps.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int64]
    lib.sfo_frame_adaptive.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_int64)]
    lib.sfo_num_substeps.restype = ctypes.c_int64
    lib.sfo_num_substeps.argtypes = [ctypes.c_void_p]
    lib.sfo_max_acc.restype = ctypes.c_double
    lib.sfo_max_acc.argtypes = [ctypes.c_void_p]
    lib.sfo_set_threads.argtypes = [ctypes.c_int]
    lib.sfo_interaction_reach.restype = ctypes.c_double
    lib.sfo_interaction_reach.argtypes = [ctypes.POINTER(SfParams), ctypes.POINTER(SfBoundaryParams)]
    for name in ("sfo_set_tangent", "sfo_get_tangent"):
        getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_int64]
    lib.sfo_seed_param.argtypes = [ctypes.c_void_p, ctypes.c_int]
    F = ctypes.POINTER(ctypes.c_float)
    lib.sfo_add_sph_particles.argtypes = [ctypes.c_void_p, F, ctypes.c_int64, F, F, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_int64]
    return lib


_ORACLE_LIB = None


def oracle_lib():
    global _ORACLE_LIB
    if _ORACLE_LIB is None:
        _ORACLE_LIB = _load_oracle()
    return _ORACLE_LIB


def set_threads(n: int) -> int:
    return oracle_lib().sfo_set_threads(int(n))


class Oracle(_Base):
    """CPU restatement of one scene. precision 32 = reference FP32 arithmetic,
    64 = the FP64 yardstick, 65 = FP64 carrying one forward-mode tangent (exact
    pathwise directional derivatives). sort_multi selects SearcherParticleType."""

    PARAMS = {"none": 0, "tan": 1, "cap": 2, "perm": 3}

    _prefix = "sfo_"

    def __init__(self, scene, precision: int = 32, sort_multi: int = 1):
        self._lib = oracle_lib()
        self.params, self.bparams, self.sparams = scene.params, scene.bparams, scene.sparams
        self._init = SceneInit(scene)
        self.n, self.nb = scene.n, scene.nb
        self.h = self._lib.sfo_create(precision, ctypes.byref(self.params), ctypes.byref(self.bparams),
                                      ctypes.byref(self.sparams), ctypes.byref(self._init.init), sort_multi)

    def set_field(self, name: str, values) -> None:
        fid, width, _ = _field_meta(name)
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        rc = self._lib.sfo_set_field(self.h, fid, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     ctypes.c_int64(self.n))
        if rc != 0:
            raise RuntimeError(f"set_field({name}) failed")

    def set_tangent(self, name: str, values) -> None:
        """Tangent of positions or velocities (precision 65), internal order."""
        fid, _, _ = _field_meta(name)
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        if self._lib.sfo_set_tangent(self.h, fid, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     ctypes.c_int64(self.n)) != 0:
            raise RuntimeError(f"set_tangent({name}) failed")

    def tangent(self, name: str) -> np.ndarray:
        fid, _, _ = _field_meta(name)
        out = np.zeros(3 * self.n, dtype=np.float64)
        if self._lib.sfo_get_tangent(self.h, fid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     ctypes.c_int64(self.n)) != 0:
            raise RuntimeError(f"tangent({name}) failed")
        return out.reshape(self.n, 3)

    def seed_param(self, which: str) -> None:
        """Differentiate by 'tan' (tan friction angle), 'cap' (capillary scale),
        'perm' (permeability scale) or 'none' (precision 65)."""
        if self._lib.sfo_seed_param(self.h, self.PARAMS[which]) != 0:
            raise RuntimeError("seed_param failed")

    def stage(self, name, time_arg: float = 0.0, adaptive: bool = False) -> None:
        sid = STAGE_ID[name] if isinstance(name, str) else int(name)
        self._lib.sfo_run_stage(self.h, sid, float(time_arg), int(adaptive))

    def add_sph_particles(self, pos, col, vel, mass: float, radius: float, capacity: int) -> bool:
        """AddSphParticles (water); False when Size() + num >= capacity."""
        p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        c = np.ascontiguousarray(col, np.float32)
        v = np.ascontiguousarray(vel, np.float32)
        rc = self._lib.sfo_add_sph_particles(self.h, _fptr(p), p.shape[0], _fptr(c), _fptr(v), float(mass),
                                             float(radius), ctypes.c_int64(capacity))
        if rc == 0:
            self.n += p.shape[0]
        return rc == 0

    def substeps(self, time_arg: float, adaptive: bool = False, n: int = 1) -> None:
        self._lib.sfo_substeps(self.h, float(time_arg), int(adaptive), ctypes.c_int64(n))

    def frame_adaptive(self, render_interval: float) -> int:
        calls = ctypes.c_int64(0)
        self._lib.sfo_frame_adaptive(self.h, float(render_interval), ctypes.byref(calls))
        return calls.value

    @property
    def num_substeps(self) -> int:
        return int(self._lib.sfo_num_substeps(self.h))

    @property
    def max_acc(self) -> float:
        return float(self._lib.sfo_max_acc(self.h))


def interaction_reach(params, bparams) -> float:
    return float(oracle_lib().sfo_interaction_reach(ctypes.byref(params), ctypes.byref(bparams)))


_REF_LIB = None


def ref_lib():
    """The reference harness library, or None where it was not built."""
    global _REF_LIB
    if _REF_LIB is None and os.path.exists(REF_SO):
        lib = ctypes.CDLL(REF_SO)
        lib.sfref_create.restype = ctypes.c_void_p
        lib.sfref_create.argtypes = [ctypes.POINTER(SfParams), ctypes.POINTER(SfBoundaryParams),
                                     ctypes.POINTER(SfSolverParams), ctypes.POINTER(SfSceneInit)]
        lib.sfref_destroy.argtypes = [ctypes.c_void_p]
        lib.sfref_substeps.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int64]
        lib.sfref_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_int64]
        lib.sfref_get_cell_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                             ctypes.c_int64]
        lib.sfref_num_substeps.restype = ctypes.c_int64
        lib.sfref_num_substeps.argtypes = [ctypes.c_void_p]
        lib.sfref_world_boundary.restype = ctypes.c_int64
        lib.sfref_world_boundary.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                             ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                             ctypes.POINTER(ctypes.c_int32), ctypes.c_int64]
        lib.sfref_emitter_points.restype = ctypes.c_int64
        lib.sfref_emitter_points.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                             ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                             ctypes.POINTER(ctypes.c_float), ctypes.c_int64]
        F = ctypes.POINTER(ctypes.c_float)
        lib.sfref_shape_multi_volume.restype = ctypes.c_int64
        lib.sfref_shape_multi_volume.argtypes = [F, ctypes.c_int64, F, ctypes.c_float, F, F, ctypes.c_int,
                                                 ctypes.c_float, ctypes.c_int, F, F, F, F, F, F,
                                                 ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, F]
        lib.sfref_boundary_shape_volume.restype = ctypes.c_int64
        lib.sfref_boundary_shape_volume.argtypes = [F, ctypes.c_int64, F, ctypes.POINTER(ctypes.c_int32),
                                                    ctypes.c_int64]
        _REF_LIB = lib
    return _REF_LIB


class RefHarness(_Base):
    """The reference's own kernels run on the CPU (see oracle/ref_harness.cpp)."""

    _prefix = "sfref_"

    def __init__(self, scene):
        self._lib = ref_lib()
        if self._lib is None:
            raise RuntimeError("reference harness not built (oracle/_ref/libsfref.so)")
        self.params, self.bparams, self.sparams = scene.params, scene.bparams, scene.sparams
        self._init = SceneInit(scene)
        self.n, self.nb = scene.n, scene.nb
        self.h = self._lib.sfref_create(ctypes.byref(self.params), ctypes.byref(self.bparams),
                                        ctypes.byref(self.sparams), ctypes.byref(self._init.init))

    def substeps(self, time_arg: float, adaptive: bool = False, n: int = 1) -> None:
        self._lib.sfref_substeps(self.h, float(time_arg), int(adaptive), ctypes.c_int64(n))

    @property
    def num_substeps(self) -> int:
        return int(self._lib.sfref_num_substeps(self.h))


def ref_world_boundary(lowest, highest, particle_radius):
    lib = ref_lib()
    lo = np.asarray(lowest, np.float32)
    hi = np.asarray(highest, np.float32)
    cap = 10_000_000
    n = lib.sfref_world_boundary(_fptr(lo), _fptr(hi), float(particle_radius), None, None, 0)
    out = np.zeros((n, 3), np.float32)
    lab = np.zeros(n, np.int32)
    lib.sfref_world_boundary(_fptr(lo), _fptr(hi), float(particle_radius), _fptr(out), _iptr(lab), min(n, cap))
    return out, lab


def ref_shape_multi_volume(shape, color, density, cda0asat, amcamcp, offset_y, lowest_y, twice=False):
    """The reference's BuildSeepageflowShapeMultiVolume on shape (n, 4): a dict
    of its output arrays and sand_min_radius."""
    lib = ref_lib()
    sh = np.ascontiguousarray(shape, np.float32)
    n = len(sh) * (2 if twice else 1)
    out = {"pos": np.zeros((n, 3), np.float32), "col": np.zeros((n, 3), np.float32),
           "cda0asat": np.zeros((n, 3), np.float32), "radius": np.zeros(n, np.float32),
           "mass": np.zeros(n, np.float32), "amcamcp": np.zeros((n, 2), np.float32),
           "label": np.zeros(n, np.int32)}
    smr = ctypes.c_float()
    c = np.asarray(color, np.float32)
    cda = np.asarray(cda0asat, np.float32)
    amc = np.asarray(amcamcp, np.float32)
    cnt = lib.sfref_shape_multi_volume(_fptr(sh), len(sh), _fptr(c), float(density), _fptr(cda), _fptr(amc),
                                       int(offset_y), float(lowest_y), int(twice), _fptr(out["pos"]),
                                       _fptr(out["col"]), _fptr(out["cda0asat"]), _fptr(out["radius"]),
                                       _fptr(out["mass"]), _fptr(out["amcamcp"]), _iptr(out["label"]), n,
                                       ctypes.byref(smr))
    assert cnt == n
    out["sand_min_radius"] = np.float32(smr.value)
    return out


def ref_boundary_shape_volume(shape):
    lib = ref_lib()
    sh = np.ascontiguousarray(shape, np.float32)
    out = np.zeros((len(sh), 3), np.float32)
    lab = np.zeros(len(sh), np.int32)
    lib.sfref_boundary_shape_volume(_fptr(sh), len(sh), _fptr(out), _iptr(lab), len(sh))
    return out, lab


def ref_emitter_points(pos, vel, kind, particle_radius, r_or_w, h=0.0):
    lib = ref_lib()
    p = np.asarray(pos, np.float32)
    v = np.asarray(vel, np.float32)
    n = lib.sfref_emitter_points(_fptr(p), _fptr(v), int(kind), float(particle_radius), float(r_or_w), float(h),
                                 None, 0)
    out = np.zeros((n, 3), np.float32)
    lib.sfref_emitter_points(_fptr(p), _fptr(v), int(kind), float(particle_radius), float(r_or_w), float(h),
                             _fptr(out), n)
    return out


_REF_GPU_LIB = None


def ref_gpu_lib():
    """The reference's CUDA library with its driver, or None where it was not built."""
    global _REF_GPU_LIB
    if _REF_GPU_LIB is None and os.path.exists(REF_GPU_SO):
        lib = ctypes.CDLL(REF_GPU_SO)
        lib.sfrg_create.restype = ctypes.c_void_p
        lib.sfrg_create.argtypes = [ctypes.POINTER(SfParams), ctypes.POINTER(SfBoundaryParams),
                                    ctypes.POINTER(SfSolverParams), ctypes.POINTER(SfSceneInit), ctypes.c_int64,
                                    ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        lib.sfrg_destroy.argtypes = [ctypes.c_void_p]
        lib.sfrg_update.restype = ctypes.c_float
        lib.sfrg_update.argtypes = [ctypes.c_void_p, ctypes.c_float]
        lib.sfrg_run.restype = ctypes.c_double
        lib.sfrg_run.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_int64]
        lib.sfrg_num_substeps.restype = ctypes.c_int64
        lib.sfrg_num_substeps.argtypes = [ctypes.c_void_p]
        lib.sfrg_size.restype = ctypes.c_int64
        lib.sfrg_size.argtypes = [ctypes.c_void_p]
        lib.sfrg_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_int64]
        lib.sfrg_get_cell_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                            ctypes.c_int64]
        _REF_GPU_LIB = lib
    return _REF_GPU_LIB


class RefGpu(_Base):
    """The reference's own CUDA library (-use_fast_math, its kernels and
    Thrust calls) driven through its public classes: each step is one
    CudaBaseSystem::UpdateSystem(render_interval) call."""

    _prefix = "sfrg_"

    EMIT_TYPES = {"square": 0, "circle": 1, "rectangle": 2}

    def __init__(self, scene, capacity=None, sort_multi: int = 1, emitter=None):
        """emitter: None, or a dict with pos, vel, col, type ('square',
        'circle', 'rectangle'), radius, width, height."""
        self._lib = ref_gpu_lib()
        if self._lib is None:
            raise RuntimeError("reference CUDA library not built (baseline/_ref/libsfrefgpu.so)")
        self.params, self.bparams, self.sparams = scene.params, scene.bparams, scene.sparams
        self._init = SceneInit(scene)
        self.n, self.nb = scene.n, scene.nb
        self._emit = None
        if emitter is not None:
            e = emitter
            self._emit = np.array(list(e["pos"]) + list(e["vel"]) + list(e["col"]) +
                                  [self.EMIT_TYPES[e.get("type", "square")], e.get("radius", 0.0),
                                   e.get("width", 0.0), e.get("height", 0.0)], np.float32)
        self.h = self._lib.sfrg_create(ctypes.byref(self.params), ctypes.byref(self.bparams),
                                       ctypes.byref(self.sparams), ctypes.byref(self._init.init),
                                       ctypes.c_int64(capacity or scene.n), int(sort_multi),
                                       _fptr(self._emit))
        if not self.h:
            raise RuntimeError("the reference CUDA library failed to build the system")

    def update(self, render_interval: float) -> float:
        """One UpdateSystem call; returns the reference's own event-timed ms."""
        ms = float(self._lib.sfrg_update(self.h, float(render_interval)))
        self.n = int(self._lib.sfrg_size(self.h))
        return ms

    def boundary_keys(self) -> np.ndarray:
        out = np.zeros(self.nb, dtype=np.float64)
        if self._lib.sfrg_get_field(self.h, 35, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    ctypes.c_int64(self.nb)) != 0:
            raise RuntimeError("boundary keys")
        return out.astype(np.int64)

    def run(self, render_interval: float, calls: int) -> float:
        """`calls` UpdateSystem calls; wall milliseconds of all of them."""
        ms = float(self._lib.sfrg_run(self.h, float(render_interval), ctypes.c_int64(calls)))
        self.n = int(self._lib.sfrg_size(self.h))
        return ms

    @property
    def num_substeps(self) -> int:
        return int(self._lib.sfrg_num_substeps(self.h))


PARTIO_SO = os.path.join(HERE, "_ref", "libpartioref.so")
_PARTIO_LIB = None


def partio_lib():
    """partio's own .bgeo writer / reader (oracle/partio_harness.cpp), or None
    where the reference sources were not mounted to build it."""
    global _PARTIO_LIB
    if _PARTIO_LIB is None and os.path.exists(PARTIO_SO):
        lib = ctypes.CDLL(PARTIO_SO)
        F = ctypes.POINTER(ctypes.c_float)
        lib.sfpartio_write.restype = ctypes.c_int
        lib.sfpartio_write.argtypes = [ctypes.c_char_p, F, F, F, ctypes.POINTER(ctypes.c_int64), ctypes.c_int64]
        lib.sfpartio_read.restype = ctypes.c_int64
        lib.sfpartio_read.argtypes = [ctypes.c_char_p, F, ctypes.c_int64, ctypes.c_int]
        _PARTIO_LIB = lib
    return _PARTIO_LIB


def partio_write(path, pos, col, radius, label) -> None:
    """The reference's ExportBgeoFileCUDA particle set written by partio."""
    lib = partio_lib()
    p = np.ascontiguousarray(pos, np.float32)
    c = np.ascontiguousarray(col, np.float32)
    r = np.ascontiguousarray(radius, np.float32)
    lab = np.ascontiguousarray(label, np.int64)
    if lib.sfpartio_write(str(path).encode(), _fptr(p), _fptr(c), _fptr(r),
                          lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(r)) != 0:
        raise RuntimeError("partio writeBGEO failed")


def partio_read_for_gpu(path, flip_yz: bool = False) -> np.ndarray:
    """ReadBgeoFileForGPU through partio's reader: (n, 4) x, y, z, pscale."""
    lib = partio_lib()
    n = lib.sfpartio_read(str(path).encode(), None, 0, int(flip_yz))
    if n < 0:
        raise RuntimeError("partio readBGEO failed")
    out = np.zeros((n, 4), np.float32)
    lib.sfpartio_read(str(path).encode(), _fptr(out), n, int(flip_yz))
    return out

"""ctypes binding of the C ABI (include/sf_capi.h) and a small Python host API
over it. The CUDA library is required: every entry point raises when
libsf_gb300.so is missing or fails to load; there is no CPU fallback.

:class:`Simulation` mirrors the reference's host-side use of ``CudaSFSystem``
(seepage_flows_cuda/src/kiri_pbs_cuda/system/cuda_sf_system.cu): construct it
from scenes (particle and boundary vectors plus parameter structs), call
:meth:`Simulation.step` as ``UpdateSystem``, read fields like the
``CudaSFParticles::Get*Ptr`` getters.
"""

from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from .params import BFIELDS, FIELDS, STAGE_ID, SfBoundaryParams, SfParams, SfSceneInit, SfSolverParams

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsf_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "sf_capi.h")

SF_OK = 0
STATUS = {0: "SF_OK", 1: "SF_ERR_INVALID", 2: "SF_ERR_CUDA", 3: "SF_ERR_CAPACITY", 4: "SF_ERR_DEVICE",
          5: "SF_ERR_NO_DEVICE", 6: "SF_ERR_UNSUPPORTED"}
ORDER = {"sorted": 0, "id": 1}

_LIB = None


class SfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def header_functions() -> list:
    """Names of the functions include/sf_capi.h declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(sf_\w+)\(", text, flags=re.M)))


def load(path: str = LIB_PATH):
    """Load libsf_gb300.so (built by build.build_library) and declare signatures."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with sph_seepage_flows_gb300.build.build_library()")
    lib = ctypes.CDLL(path)
    H = ctypes.c_void_p
    i32, i64, f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float
    P = ctypes.POINTER
    sig = {
        "sf_version": (ctypes.c_char_p, []),
        "sf_capi_version": (i32, []),
        "sf_device_count": (i32, []),
        "sf_create": (i32, [P(SfParams), P(SfBoundaryParams), P(SfSolverParams), P(SfSceneInit), i64, H, P(H)]),
        "sf_create_batched": (i32, [i32, P(SfParams), P(SfBoundaryParams), P(SfSolverParams), P(SfSceneInit),
                                    P(i64), H, P(H)]),
        "sf_destroy": (i32, [H]),
        "sf_set_params": (i32, [H, i32, P(SfParams)]),
        "sf_get_params": (i32, [H, i32, P(SfParams)]),
        "sf_step": (i32, [H, f32, P(i64), P(f32)]),
        "sf_substeps_fixed": (i32, [H, f32, i64]),
        "sf_reset_order": (i32, [H]),
        "sf_frame_adaptive": (i32, [H, f32, P(i64)]),
        "sf_run_stage": (i32, [H, i32, f32, i32]),
        "sf_get_field": (i32, [H, i32, i32, i32, ctypes.c_void_p, i64, i32]),
        "sf_set_field": (i32, [H, i32, i32, i32, ctypes.c_void_p, i64, i32]),
        "sf_get_fields": (i32, [H, i32, i32, P(i32), i32, P(ctypes.c_void_p), i64, i32]),
        "sf_set_fields": (i32, [H, i32, i32, P(i32), i32, P(ctypes.c_void_p), i64, i32]),
        "sf_get_cell_table": (i32, [H, i32, i32, P(i64), i64]),
        "sf_get_grid": (i32, [H, i32, P(i32), P(i64)]),
        "sf_size": (i32, [H, i32, P(i64), P(i64)]),
        "sf_num_scenes": (i32, [H, P(i32)]),
        "sf_num_substeps": (i32, [H, i32, P(i64)]),
        "sf_add_sph_particles": (i32, [H, i32, P(f32), i64, P(f32), P(f32), f32, f32]),
        "sf_check_error": (i32, [H, P(ctypes.c_uint32)]),
        "sf_synchronize": (i32, [H]),
        "sf_launch_count": (i32, [H, P(i64)]),
        "sf_get_list_capacity": (i32, [H, P(i32), P(i64)]),
        "sf_set_tuning": (i32, [H, i32, i32]),
        "sf_set_lanes": (i32, [H, i32]),
        "sf_set_density_staging": (i32, [H, i32]),
        "sf_get_density_staging": (i32, [H, P(i32)]),
        "sf_get_tuning": (i32, [H, P(i32), P(i32), P(i32), P(i32)]),
        "sf_autotune": (i32, [H, f32, P(i32), P(i32)]),
        "sf_last_error_string": (ctypes.c_char_p, [H]),
        "sf_adjoint_run": (i32, [H, f32, i64, i64, P(f32), P(f32), P(f32), P(f32), P(f32), P(f32)]),
        "sf_set_adjoint_seed_scale": (i32, [H, i32, f32]),
        "sf_cell_sort_noalloc": (i32, [P(SfBoundaryParams), ctypes.c_void_p, i64, ctypes.c_void_p, ctypes.c_void_p,
                                       H]),
        "sf_export_bgeo": (i32, [H, i32, ctypes.c_char_p, ctypes.c_char_p]),
        "sf_export_bgeo_device": (i32, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, i64, H]),
        "sf_read_bgeo": (i32, [ctypes.c_char_p, i32, P(f32), i64, P(i64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def device_count() -> int:
    return int(load().sf_device_count())


def _global_error() -> str:
    return (load().sf_last_error_string(None) or b"").decode()


def read_bgeo(path: str, flip_yz: bool = False) -> np.ndarray:
    """sf_read_bgeo (ReadBgeoFileForGPU): (n, 4) float32 of x, y, z, pscale."""
    lib = load()
    n = ctypes.c_int64()
    if lib.sf_read_bgeo(path.encode(), int(flip_yz), None, 0, ctypes.byref(n)) != SF_OK:
        raise RuntimeError(_global_error())
    out = np.empty((n.value, 4), np.float32)
    if lib.sf_read_bgeo(path.encode(), int(flip_yz), _fptr(out), n.value, ctypes.byref(n)) != SF_OK:
        raise RuntimeError(_global_error())
    return out


def export_bgeo_device(folder: str, name: str, pos3_ptr: int, col3_ptr: int, radius_ptr: int, label_ptr: int,
                       n: int, stream: int = 0):
    """sf_export_bgeo_device (ExportBgeoFileCUDA): device pointers to float3
    positions and colours, float radii and 64-bit labels of n particles."""
    st = load().sf_export_bgeo_device(folder.encode(), name.encode(), ctypes.c_void_p(pos3_ptr),
                                      ctypes.c_void_p(col3_ptr), ctypes.c_void_p(radius_ptr),
                                      ctypes.c_void_p(label_ptr), int(n), ctypes.c_void_p(stream or None))
    if st != SF_OK:
        raise RuntimeError(_global_error())


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if a is not None else None


class _Init:
    def __init__(self, scene):
        self.keep = {}
        for k in ("pos", "vel", "col", "mass", "radius", "cda0asat", "amcamcp", "bpos"):
            self.keep[k] = np.ascontiguousarray(getattr(scene, k), dtype=np.float32)
        for k in ("label", "blabel"):
            self.keep[k] = np.ascontiguousarray(getattr(scene, k), dtype=np.int32)
        a = self.keep
        self.s = SfSceneInit(n=scene.n, pos=_fptr(a["pos"]), vel=_fptr(a["vel"]), col=_fptr(a["col"]),
                             label=_iptr(a["label"]), mass=_fptr(a["mass"]), radius=_fptr(a["radius"]),
                             cda0asat=_fptr(a["cda0asat"]), amcamcp=_fptr(a["amcamcp"]), nb=scene.nb,
                             bpos=_fptr(a["bpos"]), blabel=_iptr(a["blabel"]))


class Simulation:
    """One handle over one or more scenes (a list gives the batched layout)."""

    def __init__(self, scenes, capacity=None, stream=None):
        self.lib = load()
        single = not isinstance(scenes, (list, tuple))
        self.scenes = [scenes] if single else list(scenes)
        ns = len(self.scenes)
        self._inits = [_Init(s) for s in self.scenes]
        if capacity is None:
            caps = [s.n for s in self.scenes]
        elif isinstance(capacity, (list, tuple)):
            caps = list(capacity)
        else:
            caps = [int(capacity)] * ns
        self.params = (SfParams * ns)(*[s.params for s in self.scenes])
        self.bparams = (SfBoundaryParams * ns)(*[s.bparams for s in self.scenes])
        self.sparams = (SfSolverParams * ns)(*[s.sparams for s in self.scenes])
        inits = (SfSceneInit * ns)(*[i.s for i in self._inits])
        caps_arr = (ctypes.c_int64 * ns)(*caps)
        h = ctypes.c_void_p()
        st = self.lib.sf_create_batched(ns, self.params, self.bparams, self.sparams, inits, caps_arr,
                                        ctypes.c_void_p(stream) if stream else None, ctypes.byref(h))
        if st != SF_OK:
            raise SfError(st, self.lib.sf_last_error_string(None).decode())
        self.h = h

    # ------------------------------------------------------------ helpers
    def _check(self, st):
        if st != SF_OK:
            raise SfError(st, self.lib.sf_last_error_string(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.sf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self, scene: int = 0) -> int:
        n = ctypes.c_int64()
        cap = ctypes.c_int64()
        self._check(self.lib.sf_size(self.h, scene, ctypes.byref(n), ctypes.byref(cap)))
        return n.value

    # ------------------------------------------------------------- stepping
    def step(self, render_interval: float, timed: bool = False):
        """UpdateSystem(render_interval): one substep with the CFL count."""
        nsub = ctypes.c_int64()
        ms = ctypes.c_float()
        self._check(self.lib.sf_step(self.h, float(render_interval), ctypes.byref(nsub),
                                     ctypes.byref(ms) if timed else None))
        return (nsub.value, ms.value) if timed else nsub.value

    def substeps_fixed(self, dt: float, n: int):
        self._check(self.lib.sf_substeps_fixed(self.h, float(dt), int(n)))

    def reset_order(self):
        """sf_reset_order: every scene's particles back in creation order, so
        that a state reset by id repeats a fresh handle's run bit for bit."""
        self._check(self.lib.sf_reset_order(self.h))

    def frame_adaptive(self, render_interval: float) -> int:
        calls = ctypes.c_int64()
        self._check(self.lib.sf_frame_adaptive(self.h, float(render_interval), ctypes.byref(calls)))
        return calls.value

    def stage(self, name, time_arg: float = 0.0, adaptive: bool = False):
        sid = STAGE_ID[name] if isinstance(name, str) else int(name)
        self._check(self.lib.sf_run_stage(self.h, sid, float(time_arg), int(adaptive)))

    def num_substeps(self, scene: int = 0) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.sf_num_substeps(self.h, scene, ctypes.byref(v)))
        return v.value

    def synchronize(self):
        self._check(self.lib.sf_synchronize(self.h))

    def launches(self) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.sf_launch_count(self.h, ctypes.byref(v)))
        return v.value

    def export_bgeo(self, folder: str, name: str, scene: int = 0):
        """sf_export_bgeo: folder/name.bgeo with position, Cd, pscale, label in the current order."""
        self._check(self.lib.sf_export_bgeo(self.h, scene, folder.encode(), name.encode()))

    def list_capacity(self) -> tuple:
        """sf_get_list_capacity: (neighbour list capacity, times the handle grew it)."""
        cap, growths = ctypes.c_int32(), ctypes.c_int64()
        self._check(self.lib.sf_get_list_capacity(self.h, ctypes.byref(cap), ctypes.byref(growths)))
        return cap.value, growths.value

    def check_error(self) -> int:
        v = ctypes.c_uint32()
        st = self.lib.sf_check_error(self.h, ctypes.byref(v))
        if st not in (SF_OK, 4):
            self._check(st)
        return v.value

    def set_params(self, params: SfParams, scene: int = 0):
        self._check(self.lib.sf_set_params(self.h, scene, ctypes.byref(params)))

    # --------------------------------------------------------------- fields
    def field(self, name: str, order: str = "sorted", scene: int = 0, out=None) -> np.ndarray:
        """Copy a field to host memory (out: optional preallocated array)."""
        fid, width, dt = FIELDS[name] if name in FIELDS else BFIELDS[name]
        n = self.scenes[scene].nb if name in BFIELDS else self.size(scene)
        shape = (n, width) if width > 1 else (n,)
        if out is None:
            out = np.empty(shape, dtype=dt)
        self._check(self.lib.sf_get_field(self.h, scene, fid, ORDER[order], out.ctypes.data_as(ctypes.c_void_p),
                                          n, 0))
        return out

    def field_device(self, name: str, dst_ptr: int, order: str = "sorted", scene: int = 0):
        fid, _, _ = FIELDS[name]
        self._check(self.lib.sf_get_field(self.h, scene, fid, ORDER[order], ctypes.c_void_p(dst_ptr),
                                          self.size(scene), 1))

    def set_field(self, name: str, values, order: str = "sorted", scene: int = 0):
        fid, width, dt = FIELDS[name]
        a = np.ascontiguousarray(values, dtype=dt)
        self._check(self.lib.sf_set_field(self.h, scene, fid, ORDER[order], a.ctypes.data_as(ctypes.c_void_p),
                                          self.size(scene), 0))

    def get_fields(self, outs: dict, order: str = "sorted", scene: int = 0):
        """sf_get_fields: {name: preallocated host array} filled in one call (one wait)."""
        names = list(outs)
        ids = (ctypes.c_int32 * len(names))(*[FIELDS[k][0] for k in names])
        ptrs = (ctypes.c_void_p * len(names))(*[outs[k].ctypes.data for k in names])
        self._check(self.lib.sf_get_fields(self.h, scene, len(names), ids, ORDER[order], ptrs, self.size(scene), 0))
        return outs

    def set_fields(self, values: dict, order: str = "sorted", scene: int = 0):
        """sf_set_fields: {name: host array} written in one call (one wait)."""
        arrs = {k: np.ascontiguousarray(v, dtype=FIELDS[k][2]) for k, v in values.items()}
        names = list(arrs)
        ids = (ctypes.c_int32 * len(names))(*[FIELDS[k][0] for k in names])
        ptrs = (ctypes.c_void_p * len(names))(*[arrs[k].ctypes.data for k in names])
        self._check(self.lib.sf_set_fields(self.h, scene, len(names), ids, ORDER[order], ptrs, self.size(scene), 0))

    def fields(self, names=None, order: str = "sorted", scene: int = 0) -> dict:
        return {k: self.field(k, order, scene) for k in (names or list(FIELDS.keys()))}

    def cell_table(self, which: int = 0, scene: int = 0) -> np.ndarray:
        g = (ctypes.c_int32 * 3)()
        nc = ctypes.c_int64()
        self._check(self.lib.sf_get_grid(self.h, scene, g, ctypes.byref(nc)))
        out = np.empty(nc.value + 1, dtype=np.int64)
        self._check(self.lib.sf_get_cell_table(self.h, scene, which,
                                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), out.size))
        return out

    def set_tuning(self, block_size: int, items_per_thread: int = 0):
        self._check(self.lib.sf_set_tuning(self.h, int(block_size), int(items_per_thread)))

    def set_lanes(self, lanes: int):
        """sf_set_lanes: threads per particle of the neighbour passes (0 = automatic)."""
        self._check(self.lib.sf_set_lanes(self.h, int(lanes)))

    def autotune(self, dt: float) -> dict:
        """sf_autotune: list capacity and per-pass block sizes for the current state."""
        bs = (ctypes.c_int32 * 6)()
        cap = ctypes.c_int32()
        self._check(self.lib.sf_autotune(self.h, float(dt), bs, ctypes.byref(cap)))
        names = ["density", "avgflow", "voidage_adhesion", "sand_momentum", "water_momentum", "integrate"]
        return {"block_sizes": dict(zip(names, list(bs))), "list_capacity": cap.value, **self.tuning()}

    def tuning(self) -> dict:
        """sf_get_tuning: threads per particle of the neighbour passes, keys per
        thread of the sort tiles and bits per radix digit currently in use."""
        lanes, items, digit = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.sf_get_tuning(self.h, None, ctypes.byref(lanes), ctypes.byref(items),
                                           ctypes.byref(digit)))
        return {"lanes": lanes.value, "sort_items": items.value, "sort_digit_bits": digit.value,
                "density_staged": self.density_staging()}

    def set_density_staging(self, staged: bool):
        """sf_set_density_staging: the one-lane density pass tests its
        candidates from a shared-memory copy of its block's stencil columns."""
        self._check(self.lib.sf_set_density_staging(self.h, int(bool(staged))))

    def density_staging(self) -> int:
        v = ctypes.c_int32()
        self._check(self.lib.sf_get_density_staging(self.h, ctypes.byref(v)))
        return v.value

    # -------------------------------------------------------------- adjoint
    def adjoint(self, dt: float, n_substeps: int, target, checkpoint_every: int | None = None,
                want_state_grads: bool = True) -> dict:
        """Runs n_substeps at the fixed dt and back-propagates the per-scene loss
        mean_sand |x_T - target|^2 (sf_adjoint_run). target: (sum n, 3), scene-major,
        id order. checkpoint_every: substeps stored per segment (default: all,
        no recomputation). Returns loss (n_scenes,), grad_params (n_scenes, 3: tan
        friction angle, capillary scale, permeability scale), grad_pos0 /
        grad_vel0 (sum n, 3, id order) and the forward / reverse device milliseconds."""
        if checkpoint_every is None:
            checkpoint_every = n_substeps
        ns = len(self.scenes)
        total = sum(self.size(s) for s in range(ns))
        tgt = np.ascontiguousarray(target, dtype=np.float32).reshape(-1)
        if tgt.size != 3 * total:
            raise ValueError(f"target must hold {total} x 3 floats")
        loss = np.zeros(ns, np.float32)
        gp = np.zeros((ns, 3), np.float32)
        gx = np.zeros((total, 3), np.float32) if want_state_grads else None
        gv = np.zeros((total, 3), np.float32) if want_state_grads else None
        ms = np.zeros(2, np.float32)
        self._check(self.lib.sf_adjoint_run(self.h, float(dt), int(n_substeps), int(checkpoint_every), _fptr(tgt),
                                            _fptr(loss), _fptr(gp), _fptr(gx), _fptr(gv), _fptr(ms)))
        return {"loss": loss, "grad_params": gp, "grad_pos0": gx, "grad_vel0": gv,
                "ms_forward": float(ms[0]), "ms_reverse": float(ms[1])}

    def set_adjoint_seed_scale(self, scale: float, scene: int = 0):
        """sf_set_adjoint_seed_scale: the scene's adjoint cotangents are seeded
        with scale x dL/dx and the returned gradients divided by it."""
        self._check(self.lib.sf_set_adjoint_seed_scale(self.h, int(scene), float(scale)))

    def add_sph_particles(self, pos, col, vel, mass: float, radius: float, scene: int = 0):
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        c = np.ascontiguousarray(col, dtype=np.float32)
        v = np.ascontiguousarray(vel, dtype=np.float32)
        self._check(self.lib.sf_add_sph_particles(self.h, scene, _fptr(p), p.shape[0], _fptr(c), _fptr(v),
                                                  float(mass), float(radius)))
        self.scenes[scene].meta["added"] = self.scenes[scene].meta.get("added", 0) + p.shape[0]

"""Python binding of libpbf_gb300.so (ctypes over include/pbf_capi.h).

The class ``Simulation`` keeps the method names of the reference's C++
``Simulation`` (src/Simulation.hpp:105-128): ``InitBuffers``, ``InitCells``,
``LoadForceMasks``, ``InitKernels`` and ``Step``; ``load_parameters`` is the
reference's ``LoadParameters`` (src/ParamUtils.cpp:24-100).  Errors raise
``PbfError`` with the library's message.  The library must have been built
(``build.py``); nothing here falls back to another implementation.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_bool, c_char_p, c_float, c_int, c_size_t, c_uint, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
# PBF_CHECK_BOUNDS=1 selects the bounds-checked build of the same sources
# (build.py --checked): indices read from device memory are checked before
# use and reported through the error word.
LIB_PATH = PKG / ("libpbf_gb300_checked.so" if os.environ.get("PBF_CHECK_BOUNDS") == "1" else "libpbf_gb300.so")

PBF_OK = 0
PBF_ERR_INVALID = -1
PBF_ERR_CUDA = -2
PBF_ERR_STATE = -3
PBF_ERR_UNSUPPORTED = -4
PBF_ERR_DEVICE_FLAG = -5
PBF_ERR_NO_DEVICE = -6
MAX_PARTICLES = 1 << 26

PAD_KEY = 2147483646
LAUNCH_SHAPE_FIELDS = 8  # PBF_LAUNCH_SHAPE_FIELDS
EMPTY = 0xFFFFFFFF


class PbfParameters(ctypes.Structure):
    """Mirror of PbfParameters (include/pbf_params.h); the prefix up to
    EnableCachedBuffers is the reference's struct Parameters."""
    _fields_ = [
        ("resetSimOnChange", c_int), ("particleCount", c_uint),
        ("xMin", c_float), ("xMax", c_float), ("yMin", c_float), ("yMax", c_float),
        ("zMin", c_float), ("zMax", c_float),
        ("waveGenAmp", c_float), ("waveGenFreq", c_float), ("waveGenDuty", c_float),
        ("timeStep", c_float), ("simIterations", c_uint), ("subSteps", c_uint),
        ("h", c_float), ("restDensity", c_float), ("epsilon", c_float), ("garvity", c_float),
        ("vorticityFactor", c_float), ("viscosityFactor", c_float),
        ("surfaceTenstionK", c_float), ("surfaceTenstionDist", c_float),
        ("friendsCircles", c_uint), ("particlesPerCircle", c_uint), ("gridBufSize", c_uint),
        ("setupSpacing", c_float), ("segmentSize", c_uint), ("sortIterations", c_uint),
        ("particleRenderSize", c_float), ("h_2", c_float), ("EnableCachedBuffers", c_bool),
        ("gravityVectorEnable", c_int), ("gravityX", c_float), ("gravityY", c_float), ("gravityZ", c_float),
        ("boxClamp", c_int), ("zeroDistanceGuard", c_int), ("relaxedMath", c_int), ("completeNeighbours", c_int),
    ]

    def copy(self) -> "PbfParameters":
        out = PbfParameters()
        ctypes.memmove(ctypes.byref(out), ctypes.byref(self), ctypes.sizeof(self))
        return out

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# PbfForceQuad (include/pbf_params.h) as a numpy record.
QUAD_DTYPE = np.dtype([("B", "<f4", 3), ("E0", "<f4", 3), ("E1", "<f4", 3), ("maskYOffset", "<i4"),
                       ("maskHeight", "<i4")])


class PbfCamera(ctypes.Structure):
    """PbfCamera (include/pbf_params.h): the renderer's camera, column-major matrices."""
    _fields_ = [("modelView", c_float * 16), ("invModelView", c_float * 16), ("projection", c_float * 16),
                ("invFocalLen", c_float * 2), ("depthRange", c_float * 2), ("widthOfNearPlane", c_float),
                ("pointSize", c_float), ("width", ctypes.c_int32), ("height", ctypes.c_int32)]


def render_camera(eye, at, up=(0.0, 1.0, 0.0), fovy_deg: float = 45.0, width: int = 640, height: int = 480,
                  point_size: float = 1.0) -> PbfCamera:
    """The reference's camera (lookAt + perspective, src/visual/visual.cpp:108-127)."""
    cam = PbfCamera()
    f3 = c_float * 3
    _check(library().pbf_render_camera(f3(*eye), f3(*at), f3(*up), float(fovy_deg), int(width), int(height),
                                       float(point_size), ctypes.byref(cam)))
    return cam


class PbfPerfTracker(ctypes.Structure):
    """PbfPerfTracker (include/pbf_capi.h): the reference's PM_PERFORMANCE_TRACKER fields."""
    _fields_ = [("eventName", ctypes.c_char * 48), ("time_start", c_uint64), ("time_end", c_uint64),
                ("total_time", ctypes.c_double), ("last_time", ctypes.c_double)]


class PbfError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


_lib = None


def library() -> ctypes.CDLL:
    """Load libpbf_gb300.so; raise when it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FileNotFoundError(f"{LIB_PATH} is not built; run position-based-fluids_gb300/build.py"
                                f"{' --checked' if 'checked' in LIB_PATH.name else ''}")
    lib = ctypes.CDLL(str(LIB_PATH))
    P = POINTER(PbfParameters)
    f32p, u32p = POINTER(c_float), POINTER(c_uint32)
    sig = {
        "pbf_default_parameters": [P],
        "pbf_load_parameters": [c_char_p, P, POINTER(c_int)],
        "pbf_create": [P, c_int, POINTER(c_void_p)],
        "pbf_destroy": [c_void_p],
        "pbf_init_buffers": [c_void_p, f32p, f32p],
        "pbf_init_cells": [c_void_p],
        "pbf_load_force_masks": [c_void_p, u32p, c_int, c_int],
        "pbf_init_kernels": [c_void_p],
        "pbf_set_params": [c_void_p, P],
        "pbf_set_pause": [c_void_p, c_int],
        "pbf_step": [c_void_p, c_int],
        "pbf_step_async": [c_void_p, c_int],
        "pbf_synchronize": [c_void_p],
        "pbf_read_state": [c_void_p, c_void_p, c_void_p, c_void_p],
        "pbf_write_state": [c_void_p, c_void_p, c_void_p],
        "pbf_write_state_async": [c_void_p, c_void_p, c_void_p],
        "pbf_read_state_async": [c_void_p, c_void_p, c_void_p, c_void_p],
        "pbf_step_read_async": [c_void_p, c_int, c_void_p, c_void_p],
        "pbf_device_positions": [c_void_p, POINTER(c_void_p)],
        "pbf_get_stream": [c_void_p, POINTER(c_void_p)],
        "pbf_sort_state": [c_void_p, f32p, u32p, u32p, u32p],
        "pbf_read_friends": [c_void_p, u32p, u32p, c_int],
        "pbf_read_sort": [c_void_p, u32p, u32p, u32p],
        "pbf_enable_stage_timing": [c_void_p, c_int],
        "pbf_stage_timings": [c_void_p, f32p, c_int, POINTER(c_int), c_char_p, c_size_t],
        "pbf_launch_count": [c_void_p, POINTER(c_uint64)],
        "pbf_use_graph": [c_void_p, c_int],
        "pbf_reference_lattice": [P, f32p],
        "pbf_scene_block": [c_int, c_int, c_int, c_float, c_float, c_float, c_float, c_float, c_uint64, f32p],
        "pbf_sort_state_noalloc": [P, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
        "pbf_scene_double_dam_break": [c_int, c_float, c_float, c_float, c_uint64, f32p, f32p],
        "pbf_create_batch": [P, c_int, c_int, POINTER(c_void_p)],
        "pbf_scene_offsets": [c_void_p, u32p],
        "pbf_get_launch_shape": [c_void_p, POINTER(c_int)],
        "pbf_set_launch_shape": [c_void_p, POINTER(c_int)],
        "pbf_autotune": [c_void_p, c_int, POINTER(c_int)],
        "pbf_read_ids": [c_void_p, u32p],
        "pbf_set_force_quads": [c_void_p, c_void_p, c_int],
        "pbf_set_wave_position": [c_void_p, c_float],
        "pbf_perf_trackers": [c_void_p, c_void_p, c_int, POINTER(c_int)],
        "pbf_enable_nvtx": [c_void_p, c_int],
        "pbf_load_scene": [c_char_p, c_void_p],
        "pbf_scene_positions": [P, c_void_p, f32p],
        "pbf_render_camera": [c_void_p, c_void_p, c_void_p, c_float, c_int, c_int, c_float, c_void_p],
        "pbf_render_frame": [c_void_p, c_void_p, c_int],
        "pbf_render_read": [c_void_p, c_int, f32p],
        "pbf_perf_export_json": [c_void_p, c_char_p, c_size_t, POINTER(c_size_t)],
        "pbf_save_state": [c_void_p, ctypes.c_char_p],
        "pbf_load_state": [c_void_p, ctypes.c_char_p],
        "pbf_rollout_forward": [c_void_p, c_int, c_int],
        "pbf_rollout_backward": [c_void_p, f32p, f32p, POINTER(c_float), f32p],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = c_int
    lib.pbf_last_error.argtypes = [c_void_p]
    lib.pbf_last_error.restype = c_char_p
    lib.pbf_wave_position.argtypes = [P, c_float]
    lib.pbf_wave_position.restype = c_float
    _lib = lib
    return lib


def _check(rc: int, ctx=None) -> None:
    if rc != PBF_OK:
        msg = library().pbf_last_error(ctx).decode(errors="replace")
        raise PbfError(rc, msg)


def _f32(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_float))


def _u32(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_uint32))


def default_parameters() -> PbfParameters:
    p = PbfParameters()
    _check(library().pbf_default_parameters(ctypes.byref(p)))
    return p


def load_parameters(text: str, base: PbfParameters | None = None) -> PbfParameters:
    """LoadParameters: parse `.par` text on top of `base` (default: zeros)."""
    p = base.copy() if base is not None else default_parameters()
    unknown = c_int(0)
    _check(library().pbf_load_parameters(text.encode(), ctypes.byref(p), ctypes.byref(unknown)))
    p._unknown_keys = unknown.value  # type: ignore[attr-defined]
    return p


def load_scenario(name: str) -> PbfParameters:
    """Load one of the bundled scenario files (scenarios/<name>.par)."""
    path = PKG / "scenarios" / (name if name.endswith(".par") else name + ".par")
    return load_parameters(path.read_text())


def scene_block(nx: int, ny: int, nz: int, spacing: float, origin=(0.0, 0.0, 0.0), jitter: float = 0.0,
                seed: int = 0) -> np.ndarray:
    out = np.zeros((nx * ny * nz, 4), np.float32)
    _check(library().pbf_scene_block(nx, ny, nz, spacing, float(origin[0]), float(origin[1]), float(origin[2]),
                                     jitter, seed, _f32(out)))
    return out


def sort_state_noalloc(params: PbfParameters, d_pred: int, d_keys: int, d_perm: int, d_cells: int | None = None,
                       stream: int | None = None) -> None:
    """pbf_sort_state_noalloc on device addresses (see include/pbf_capi.h)."""
    _check(library().pbf_sort_state_noalloc(ctypes.byref(params), d_pred, d_keys, d_perm, d_cells, stream))


def wave_position(params: PbfParameters, wave_time: float) -> float:
    """The reference's wave position after `wave_time` seconds (src/Runner.cpp:103-107)."""
    return float(library().pbf_wave_position(ctypes.byref(params), float(wave_time)))


def reference_lattice(params: PbfParameters) -> np.ndarray:
    out = np.zeros((params.particleCount, 4), np.float32)
    _check(library().pbf_reference_lattice(ctypes.byref(params), _f32(out)))
    return out


class Simulation:
    """The reference's Simulation over the C-ABI, on one CUDA device."""

    def __init__(self, params, device: int = 0):
        """`params`: one PbfParameters, or a list of them for a batch of scenes."""
        self.lib = library()
        self._ctx = c_void_p()
        if isinstance(params, (list, tuple)):
            arr = (PbfParameters * len(params))(*[p.copy() for p in params])
            _check(self.lib.pbf_create_batch(arr, len(params), device, ctypes.byref(self._ctx)))
            self.scene_params = [p.copy() for p in params]
            self.params = params[0].copy()
            self.params.particleCount = sum(int(p.particleCount) for p in params)
        else:
            self.scene_params = None
            self.params = params.copy()
            _check(self.lib.pbf_create(ctypes.byref(self.params), device, ctypes.byref(self._ctx)))

    # -- lifetime ----------------------------------------------------------
    def close(self) -> None:
        if self._ctx:
            self.lib.pbf_destroy(self._ctx)
            self._ctx = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> c_void_p:
        return self._ctx

    @property
    def n(self) -> int:
        return int(self.params.particleCount)

    # -- the reference's methods --------------------------------------------
    def InitBuffers(self, pos: np.ndarray | None = None, vel: np.ndarray | None = None) -> None:
        p = None if pos is None else np.ascontiguousarray(pos, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        for a in (p, v):
            if a is not None and a.size != 4 * self.n:
                raise ValueError("state arrays must hold particleCount float4 records")
        _check(self.lib.pbf_init_buffers(self._ctx, None if p is None else _f32(p), None if v is None else _f32(v)),
               self._ctx)

    def InitCells(self) -> None:
        _check(self.lib.pbf_init_cells(self._ctx), self._ctx)

    def LoadForceMasks(self, mask: np.ndarray | None = None) -> None:
        if mask is None:
            _check(self.lib.pbf_load_force_masks(self._ctx, None, 0, 0), self._ctx)
        else:
            m = np.ascontiguousarray(mask, np.uint32)
            _check(self.lib.pbf_load_force_masks(self._ctx, _u32(m), m.shape[1], m.shape[0]), self._ctx)

    def InitKernels(self) -> bool:
        _check(self.lib.pbf_init_kernels(self._ctx), self._ctx)
        return True

    def Step(self, substeps: int = 1) -> None:
        _check(self.lib.pbf_step(self._ctx, substeps), self._ctx)

    @property
    def bPauseSim(self) -> bool:
        return bool(getattr(self, "_paused", False))

    @bPauseSim.setter
    def bPauseSim(self, value: bool) -> None:
        self._paused = bool(value)
        _check(self.lib.pbf_set_pause(self._ctx, int(self._paused)), self._ctx)

    # -- conveniences ----------------------------------------------------------
    @classmethod
    def create(cls, params: PbfParameters, pos=None, vel=None, device: int = 0) -> "Simulation":
        """Construct and run InitBuffers, InitCells, LoadForceMasks, InitKernels."""
        sim = cls(params, device)
        sim.InitBuffers(pos, vel)
        sim.InitCells()
        sim.LoadForceMasks()
        sim.InitKernels()
        return sim

    def set_params(self, params: PbfParameters) -> None:
        _check(self.lib.pbf_set_params(self._ctx, ctypes.byref(params)), self._ctx)
        self.params = params.copy()

    def step_async(self, substeps: int = 1) -> None:
        _check(self.lib.pbf_step_async(self._ctx, substeps), self._ctx)

    def synchronize(self) -> None:
        _check(self.lib.pbf_synchronize(self._ctx), self._ctx)

    def read_state(self):
        pos = np.empty((self.n, 4), np.float32)
        vel = np.empty((self.n, 4), np.float32)
        pred = np.empty((self.n, 4), np.float32)
        _check(self.lib.pbf_read_state(self._ctx, pos.ctypes.data, vel.ctypes.data, pred.ctypes.data), self._ctx)
        return pos, vel, pred

    def read_state_into(self, pos_ptr: int | None, vel_ptr: int | None = None, pred_ptr: int | None = None) -> None:
        _check(self.lib.pbf_read_state(self._ctx, pos_ptr, vel_ptr, pred_ptr), self._ctx)

    def write_state(self, pos: np.ndarray | None = None, vel: np.ndarray | None = None) -> None:
        p = None if pos is None else np.ascontiguousarray(pos, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        _check(self.lib.pbf_write_state(self._ctx, None if p is None else p.ctypes.data,
                                        None if v is None else v.ctypes.data), self._ctx)

    def write_state_async(self, pos_ptr: int | None, vel_ptr: int | None = None) -> None:
        """pbf_write_state_async from host addresses (page-locked for overlap)."""
        _check(self.lib.pbf_write_state_async(self._ctx, pos_ptr, vel_ptr), self._ctx)

    def read_state_async(self, pos_ptr: int | None, vel_ptr: int | None = None, pred_ptr: int | None = None) -> None:
        _check(self.lib.pbf_read_state_async(self._ctx, pos_ptr, vel_ptr, pred_ptr), self._ctx)

    def step_read_async(self, substeps: int, pos_ptr: int | None, vel_ptr: int | None = None) -> None:
        """Step and copy positions / velocities to host addresses; the
        position copy overlaps the last substep's XSPH and vorticity."""
        _check(self.lib.pbf_step_read_async(self._ctx, substeps, pos_ptr, vel_ptr), self._ctx)

    def write_state_from(self, pos_ptr: int | None, vel_ptr: int | None = None) -> None:
        _check(self.lib.pbf_write_state(self._ctx, pos_ptr, vel_ptr), self._ctx)

    def sort_state(self, pred: np.ndarray):
        """Keys, permutation (IntCeil(N, 2048) entries) and cell table from `pred`."""
        pred = np.ascontiguousarray(pred, np.float32)
        nkeys = (self.n + 2047) // 2048 * 2048
        keys = np.empty(nkeys, np.uint32)
        perm = np.empty(nkeys, np.uint32)
        cells = np.empty(2 * self.params.gridBufSize, np.uint32)
        _check(self.lib.pbf_sort_state(self._ctx, _f32(pred), _u32(keys), _u32(perm), _u32(cells)), self._ctx)
        return keys, perm, cells

    def read_sort(self):
        """Keys and permutation (IntCeil(N, 2048) entries) and the cell table
        of the last substep, as the pipeline computed them."""
        nkeys = (self.n + 2047) // 2048 * 2048
        keys = np.empty(nkeys, np.uint32)
        perm = np.empty(nkeys, np.uint32)
        scenes = len(self.scene_params) if self.scene_params else 1
        cells = np.empty(2 * self.params.gridBufSize * scenes, np.uint32)
        _check(self.lib.pbf_read_sort(self._ctx, _u32(keys), _u32(perm), _u32(cells)), self._ctx)
        return keys, perm, cells

    def read_friends(self, slots: int | None = None):
        """(counts[N,2], list[slots,N]) of the last substep."""
        if slots is None:
            slots = int(self.params.friendsCircles * self.params.particlesPerCircle)
        counts = np.empty((self.n, 2), np.uint32)
        lst = np.zeros((slots, self.n), np.uint32)
        _check(self.lib.pbf_read_friends(self._ctx, _u32(counts), _u32(lst), slots), self._ctx)
        return counts, lst

    def device_positions(self) -> int:
        p = c_void_p()
        _check(self.lib.pbf_device_positions(self._ctx, ctypes.byref(p)), self._ctx)
        return int(p.value or 0)

    def stream(self) -> int:
        s = c_void_p()
        _check(self.lib.pbf_get_stream(self._ctx, ctypes.byref(s)), self._ctx)
        return int(s.value or 0)

    def enable_stage_timing(self, on: bool = True) -> None:
        _check(self.lib.pbf_enable_stage_timing(self._ctx, int(on)), self._ctx)

    def stage_timings(self) -> dict:
        ms = (c_float * 64)()
        count = c_int(0)
        names = ctypes.create_string_buffer(4096)
        _check(self.lib.pbf_stage_timings(self._ctx, ms, 64, ctypes.byref(count), names, 4096), self._ctx)
        keys = names.value.decode().split("\n") if count.value else []
        return {k: float(ms[i]) for i, k in enumerate(keys)}

    def launch_count(self) -> int:
        v = c_uint64(0)
        _check(self.lib.pbf_launch_count(self._ctx, ctypes.byref(v)), self._ctx)
        return int(v.value)

    def use_graph(self, on: bool) -> None:
        _check(self.lib.pbf_use_graph(self._ctx, int(on)), self._ctx)

    def set_force_quads(self, quads) -> None:
        """Force planes: a numpy array of QUAD_DTYPE records (PbfForceQuad)."""
        q = np.ascontiguousarray(quads, QUAD_DTYPE) if quads is not None else np.zeros(0, QUAD_DTYPE)
        _check(self.lib.pbf_set_force_quads(self._ctx, q.ctypes.data if len(q) else None, len(q)), self._ctx)

    def render_frame(self, cam: PbfCamera, mode: int = 0) -> None:
        _check(self.lib.pbf_render_frame(self._ctx, ctypes.byref(cam), int(mode)), self._ctx)

    def render_read(self, cam: PbfCamera, which: int = 0) -> np.ndarray:
        """[height, width, 4] float32, row 0 at the bottom: 0 output, 1 splat, 2 smoothed depth."""
        img = np.empty((cam.height, cam.width, 4), np.float32)
        _check(self.lib.pbf_render_read(self._ctx, int(which), _f32(img)), self._ctx)
        return img

    def enable_nvtx(self, on: bool = True) -> None:
        _check(self.lib.pbf_enable_nvtx(self._ctx, int(on)), self._ctx)

    def perf_trackers(self) -> list:
        """[(eventName, time_start ns, time_end ns, total_time ms, last_time ms)] in order of first use."""
        count = c_int(0)
        _check(self.lib.pbf_perf_trackers(self._ctx, None, 0, ctypes.byref(count)), self._ctx)
        arr = (PbfPerfTracker * max(1, count.value))()
        _check(self.lib.pbf_perf_trackers(self._ctx, arr, count.value, ctypes.byref(count)), self._ctx)
        return [(t.eventName.decode(), t.time_start, t.time_end, t.total_time, t.last_time)
                for t in arr[:count.value]]

    def perf_json(self) -> str:
        need = c_size_t(0)
        _check(self.lib.pbf_perf_export_json(self._ctx, None, 0, ctypes.byref(need)), self._ctx)
        buf = ctypes.create_string_buffer(need.value)
        _check(self.lib.pbf_perf_export_json(self._ctx, buf, need.value, ctypes.byref(need)), self._ctx)
        return buf.value.decode()

    def set_wave_position(self, wave_pos: float) -> None:
        _check(self.lib.pbf_set_wave_position(self._ctx, float(wave_pos)), self._ctx)

    def save_state(self, path) -> None:
        _check(self.lib.pbf_save_state(self._ctx, str(path).encode()), self._ctx)

    def load_state(self, path) -> None:
        _check(self.lib.pbf_load_state(self._ctx, str(path).encode()), self._ctx)

    def read_ids(self) -> np.ndarray:
        ids = np.empty(self.n, np.uint32)
        _check(self.lib.pbf_read_ids(self._ctx, _u32(ids)), self._ctx)
        return ids

    def positions_by_id(self) -> np.ndarray:
        pos, _, _ = self.read_state()
        out = np.empty_like(pos)
        out[self.read_ids()] = pos
        return out

    def rollout_forward(self, substeps: int, checkpoint_every: int = 10) -> None:
        _check(self.lib.pbf_rollout_forward(self._ctx, substeps, checkpoint_every), self._ctx)

    def rollout_backward(self, dL_dx_by_id: np.ndarray):
        """(dL/dv0 [N,4] by original index, dL/d viscosityFactor, dL/d gravity [3])."""
        gx = np.ascontiguousarray(dL_dx_by_id, np.float32).reshape(self.n, 4)
        dv = np.zeros((self.n, 4), np.float32)
        dc = c_float(0)
        dg = np.zeros(3, np.float32)
        _check(self.lib.pbf_rollout_backward(self._ctx, _f32(gx), _f32(dv), ctypes.byref(dc), _f32(dg)), self._ctx)
        return dv, dc.value, dg

    def scene_offsets(self) -> np.ndarray:
        k = len(self.scene_params) if self.scene_params else 1
        out = np.zeros(k + 1, np.uint32)
        _check(self.lib.pbf_scene_offsets(self._ctx, _u32(out)), self._ctx)
        return out

    def launch_shape(self) -> list:
        """[friends, scaling, delta, viscosity, vorticity block sizes,
        friends algorithm, balance, persistent] (PBF_LAUNCH_SHAPE_FIELDS)."""
        b = (c_int * LAUNCH_SHAPE_FIELDS)()
        _check(self.lib.pbf_get_launch_shape(self._ctx, b), self._ctx)
        return list(b)

    def set_launch_shape(self, blocks) -> None:
        blocks = list(blocks)
        blocks += self.launch_shape()[len(blocks):]
        b = (c_int * LAUNCH_SHAPE_FIELDS)(*blocks)
        _check(self.lib.pbf_set_launch_shape(self._ctx, b), self._ctx)

    def autotune(self, trial_substeps: int = 2) -> list:
        b = (c_int * LAUNCH_SHAPE_FIELDS)()
        _check(self.lib.pbf_autotune(self._ctx, trial_substeps, b), self._ctx)
        return list(b)


EXPORTED_SYMBOLS = sorted(
    ["pbf_last_error"] + [
        "pbf_default_parameters", "pbf_load_parameters", "pbf_create", "pbf_destroy", "pbf_init_buffers",
        "pbf_init_cells", "pbf_load_force_masks", "pbf_init_kernels", "pbf_set_params", "pbf_set_pause",
        "pbf_step", "pbf_step_async", "pbf_synchronize", "pbf_read_state", "pbf_write_state",
        "pbf_device_positions", "pbf_get_stream", "pbf_sort_state", "pbf_read_sort", "pbf_read_friends",
        "pbf_enable_stage_timing", "pbf_stage_timings", "pbf_launch_count", "pbf_use_graph",
        "pbf_reference_lattice", "pbf_scene_block", "pbf_sort_state_noalloc", "pbf_scene_double_dam_break",
        "pbf_create_batch", "pbf_scene_offsets", "pbf_get_launch_shape", "pbf_set_launch_shape", "pbf_autotune",
        "pbf_read_ids", "pbf_rollout_forward", "pbf_rollout_backward", "pbf_set_force_quads",
        "pbf_set_wave_position", "pbf_wave_position", "pbf_save_state", "pbf_load_state",
        "pbf_perf_trackers", "pbf_perf_export_json", "pbf_render_camera", "pbf_render_frame", "pbf_render_read",
        "pbf_write_state_async", "pbf_read_state_async", "pbf_step_read_async", "pbf_enable_nvtx", "pbf_load_scene", "pbf_scene_positions",
    ])


# Dam-break scenes: scenario file + the block the particles start in.
SCENES = ("dam_break_32k", "dam_break_1m", "dam_break_32k_literal")


class PbfScene(ctypes.Structure):
    """PbfScene (include/pbf_params.h): a scenario file's initial block."""
    _fields_ = [("blockDims", ctypes.c_int32 * 3), ("blockOrigin", c_float * 3), ("jitter", c_float),
                ("seed", c_uint64)]


def load_scene(text: str) -> PbfScene:
    """pbf_load_scene: the BlockDims / BlockOrigin / Jitter / Seed keys."""
    s = PbfScene()
    _check(library().pbf_load_scene(text.encode(), ctypes.byref(s)))
    return s


def scene_positions(params: PbfParameters, scene: PbfScene) -> np.ndarray:
    n = scene.blockDims[0] * scene.blockDims[1] * scene.blockDims[2]
    out = np.zeros((n, 4), np.float32)
    _check(library().pbf_scene_positions(ctypes.byref(params), ctypes.byref(scene), _f32(out)))
    return out


def make_scene(name: str):
    """(params, pos[N,4], vel[N,4]) of a bundled scenario file: its
    parameters and its initial block (BlockDims, BlockOrigin, Jitter, Seed)."""
    text = (PKG / "scenarios" / f"{name}.par").read_text()
    params = load_parameters(text)
    pos = scene_positions(params, load_scene(text))
    if pos.shape[0] != params.particleCount:
        raise ValueError(f"scene {name}: block holds {pos.shape[0]} particles, .par says {params.particleCount}")
    return params, pos, np.zeros_like(pos)


def grid_size_for_box(box, h: float) -> int:
    """Smallest power-of-two hash size holding the Morton number of every cell
    of the box (so that the modulo never merges two cells of the box)."""
    import math
    cells = [max(1, int(math.ceil((box[2 * k + 1] - box[2 * k]) / h))) for k in range(3)]
    bits = [max(1, int(math.ceil(math.log2(c)))) if c > 1 else 1 for c in cells]
    top = max(3 * bits[0] - 3, 3 * bits[1] - 2, 3 * bits[2] - 1) + 1  # highest Morton bit + 1
    return 1 << top


def make_double_dam_break(n: int, iterations: int = 4, seed: int = 20240601, fill: float = 0.25):
    """(params, pos, vel) of the particle-count sweep's double dam break: the
    dam_break_1m solver settings in a box sized for a 25 % fill."""
    params = load_scenario("dam_break_1m")
    pos = np.zeros((n, 4), np.float32)
    box = np.zeros(6, np.float32)
    _check(library().pbf_scene_double_dam_break(n, 0.05, fill, 0.005, seed, _f32(pos), _f32(box)))
    params.particleCount = n
    params.simIterations = iterations
    params.xMin, params.xMax, params.yMin, params.yMax, params.zMin, params.zMax = (float(b) for b in box)
    params.gridBufSize = grid_size_for_box(box, params.h)
    return params, pos, np.zeros_like(pos)


def make_rollout_scene(nx: int = 64, ny: int = 32, nz: int = 32, seed: int = 20240601):
    """(params, pos, vel) of the differentiable-rollout dam break: an
    nx x ny x nz block (spacing 0.05, jitter 0.005, origin 0.025) in the low
    corner of a (2 nx, ny, nz) x 0.05 box, the dam_break_32k solver settings,
    gravity as the vector (0, -9.8, 0) so that it can be differentiated."""
    params = load_scenario("dam_break_32k")
    s = 0.05
    pos = scene_block(nx, ny, nz, s, (0.025, 0.025, 0.025), 0.005, seed)
    params.particleCount = nx * ny * nz
    box = (0.0, 2 * nx * s, 0.0, ny * s, 0.0, nz * s)
    params.xMin, params.xMax, params.yMin, params.yMax, params.zMin, params.zMax = box
    params.gridBufSize = grid_size_for_box(box, params.h)
    params.gravityVectorEnable = 1
    params.gravityX, params.gravityY, params.gravityZ = 0.0, -float(params.garvity), 0.0
    return params, pos, np.zeros_like(pos)


def rollout_target_params(params: PbfParameters, tilt_degrees: float = 5.0, xsph_c: float = 0.03) -> PbfParameters:
    """Parameters of the rollout's target run: gravity tilted by
    `tilt_degrees` towards +x and the XSPH factor c (in the units of the
    reference's ViscosityFactor times the rest density, as in the batched
    scenes: viscosityFactor = c / restDensity)."""
    import math
    p = PbfParameters.from_buffer_copy(params)
    g = float(params.garvity)
    t = math.radians(tilt_degrees)
    p.gravityVectorEnable = 1
    p.gravityX, p.gravityY, p.gravityZ = g * math.sin(t), -g * math.cos(t), 0.0
    p.viscosityFactor = xsph_c / float(params.restDensity)
    return p


def make_batch_scenes(count: int = 256, seed: int = 7, fill: float = 0.3, first: int | None = None):
    """Scenes of the batched benchmark: `count` dam breaks with particle counts
    drawn log-uniformly in [4096, 65536] (numpy PCG64 with `seed`); scene s is
    a block of n_s particles (a cubic lattice of a^3 >= n_s sites at spacing
    0.05, x fastest, cut at n_s) in the low corner of a 2:1:1 box of volume
    n_s * 0.05^3 / fill, with gravity 9.8 tilted by
    U(0, 10) degrees about a random horizontal axis and XSPH c ~ U(0.005, 0.05)
    (viscosityFactor = c / 6378, the reference's XSPH omitting 1/rho_j).
    All scenes share one gridBufSize, the largest any of them needs.
    Returns (list of PbfParameters, list of pos arrays).  `first` keeps only
    the first scenes of the same draw."""
    import math
    rng = np.random.default_rng(seed)
    counts = np.rint(np.exp(rng.uniform(math.log(4096), math.log(65536), count))).astype(int)
    tilt = np.radians(rng.uniform(0.0, 10.0, count))
    phi = rng.uniform(0.0, 2.0 * math.pi, count)
    cvis = rng.uniform(0.005, 0.05, count)
    base = load_scenario("dam_break_1m")
    scenes, positions = [], []
    for s in range(count):
        n = int(counts[s])
        side = (n * 0.05 ** 3 / fill / 2.0) ** (1.0 / 3.0)
        a = 1
        while a * a * a < n:
            a += 1
        pos = scene_block(a, a, a, 0.05, (0.025, 0.025, 0.025), 0.005, seed * 1000003 + s)[:n].copy()
        p = base.copy()
        p.particleCount = n
        p.xMin, p.xMax, p.yMin, p.yMax, p.zMin, p.zMax = 0.0, 2.0 * side, 0.0, side, 0.0, side
        g = 9.8
        p.gravityVectorEnable = 1
        p.gravityX = g * math.sin(tilt[s]) * math.sin(phi[s])
        p.gravityY = -g * math.cos(tilt[s])
        p.gravityZ = -g * math.sin(tilt[s]) * math.cos(phi[s])
        p.viscosityFactor = float(cvis[s] / 6378.0)
        scenes.append(p)
        positions.append(pos)
    grid = max(grid_size_for_box([q.xMin, q.xMax, q.yMin, q.yMax, q.zMin, q.zMax], q.h) for q in scenes)
    for q in scenes:
        q.gridBufSize = grid
    if first is not None:
        scenes, positions = scenes[:first], positions[:first]
    return scenes, positions

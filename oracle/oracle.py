"""ctypes binding of the test oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  ``step`` runs the FP32 restatement of Simulation::Step,
``step_f64`` the FP64 one, ``sort`` the key / sort / cell-table stages, and
``ref_step`` / ``ref_sort`` the reference's own kernels compiled through the
OpenCL-C shim (available where oracle/_ref was built).
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_float, c_double, c_int, c_uint32, c_void_p

import numpy as np

from . import build as _build  # noqa: F401  (package-relative when imported as oracle.oracle)


class OracleDebug(ctypes.Structure):
    _fields_ = [
        ("keys", c_void_p), ("perm", c_void_p), ("cells", c_void_p), ("counts", c_void_p),
        ("list", c_void_p), ("list_slots", c_int), ("density", c_void_p), ("lambda_", c_void_p),
        ("omega", c_void_p),
    ]


_lib = None
_ref = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        l = ctypes.CDLL(str(path))
        l.oracle_step_f32.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_int,
                                      POINTER(OracleDebug)]
        l.oracle_step_f64.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int]
        l.oracle_sort_f32.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
        l.oracle_constants.argtypes = [c_void_p, POINTER(c_float), POINTER(c_float), POINTER(c_float)]
        l.oracle_grid_hash.argtypes = [c_int, c_int, c_int, c_uint32]
        l.oracle_grid_hash.restype = c_uint32
        for f in (l.oracle_step_f32, l.oracle_step_f64, l.oracle_sort_f32, l.oracle_constants, l.oracle_max_threads):
            f.restype = c_int
        l.oracle_rollout_record.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int]
        l.oracle_rollout_record.restype = c_void_p
        l.oracle_rollout_free.argtypes = [c_void_p]
        l.oracle_rollout_replay_f64.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        l.oracle_rollout_replay_f64.restype = c_double
        l.oracle_rollout_grad_f64.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                              c_void_p]
        l.oracle_rollout_grad_f64.restype = c_double
        l.oracle_rollout_grad_f32.argtypes = [c_void_p] * 8
        l.oracle_rollout_grad_f32.restype = c_double
        l.oracle_set_force_planes.argtypes = [c_void_p, c_int, c_void_p, c_int, c_int]
        l.oracle_set_force_planes.restype = c_int
        l.oracle_set_wave_position.argtypes = [c_float]
        l.oracle_set_wave_position.restype = None
        l.oracle_render.argtypes = [c_void_p, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p, c_void_p]
        l.oracle_render.restype = c_int
        l.oracle_noise_sinf.argtypes = [c_float]
        l.oracle_noise_sinf.restype = c_float
        l.oracle_load_scenario.argtypes = [ctypes.c_char_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        l.oracle_load_scenario.restype = c_int
        l.oracle_scene_block.argtypes = [c_int, c_int, c_int, c_float, c_void_p, c_float, ctypes.c_uint64, c_void_p]
        l.oracle_scene_block.restype = c_int
        _lib = l
    return _lib


def ref_available() -> bool:
    ref = _build.reference_dir()
    return _build.REF_LIB.exists() or _build.REF_TU.exists() or (ref is not None and (ref / "assets").is_dir())


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            raise FileNotFoundError("the reference kernels are not available (oracle/_ref)")
        l = ctypes.CDLL(str(path))
        l.ref_step_f32.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]
        l.ref_sort_f32.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
        l.ref_step_f32.restype = c_int
        l.ref_sort_f32.restype = c_int
        l.ref_set_force_mask.argtypes = [c_void_p, c_int, c_int]
        l.ref_set_force_mask.restype = None
        l.ref_set_threads.argtypes = [c_int]
        l.ref_set_threads.restype = None
        l.ref_run_timed.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_double,
                                    POINTER(c_int), POINTER(c_double)]
        l.ref_run_timed.restype = c_int
        l.ref_max_threads.argtypes = []
        l.ref_max_threads.restype = c_int
        _ref = l
    return _ref


# PbfForceQuad (include/pbf_params.h) as a numpy record.
QUAD_DTYPE = np.dtype([("B", "<f4", 3), ("E0", "<f4", 3), ("E1", "<f4", 3), ("maskYOffset", "<i4"),
                       ("maskHeight", "<i4")])


def set_force_planes(quads=None, mask=None):
    """Force planes for every later oracle step (None / empty removes them);
    mask: 2-D uint32 array (rows, width) or None for the empty mask."""
    q = np.zeros(0, QUAD_DTYPE) if quads is None else np.ascontiguousarray(quads, QUAD_DTYPE)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint32)
    rc = lib().oracle_set_force_planes(_ptr(q) if len(q) else None, len(q), _ptr(m),
                                       0 if m is None else m.shape[1], 0 if m is None else m.shape[0])
    if rc != 0:
        raise ValueError("oracle_set_force_planes rejected the planes")


def ref_set_force_mask(mask=None):
    """The mask the shimmed reference computeDelta reads (its 14 planes are in its source)."""
    m = None if mask is None else np.ascontiguousarray(mask, np.uint32)
    ref().ref_set_force_mask(_ptr(m), 0 if m is None else m.shape[1], 0 if m is None else m.shape[0])


def load_scenario(text: str, params_type):
    """A scenario file's parameters and initial block, read the way the
    reference's LoadParameters reads a `.par` file (oracle_load_scenario).
    `params_type` is the ctypes mirror of PbfParameters to fill (zeroed
    first).  Returns (params, (nx, ny, nz), origin, jitter, seed)."""
    params = params_type()
    dims = np.zeros(3, np.int32)
    origin = np.zeros(3, np.float32)
    jitter = c_float(0.0)
    seed = ctypes.c_uint64(0)
    lib().oracle_load_scenario(text.encode(), ctypes.byref(params), _ptr(dims), _ptr(origin), ctypes.byref(jitter),
                               ctypes.byref(seed))
    return params, tuple(int(d) for d in dims), origin, jitter.value, seed.value


def make_scene(path, params_type):
    """(params, pos[N,4], vel[N,4]) of a scenario file with an initial block
    (BlockDims, BlockOrigin, Jitter, Seed): the same scene the product's
    scenario reader builds, made here without the product library."""
    from pathlib import Path
    params, dims, origin, jitter, seed = load_scenario(Path(path).read_text(), params_type)
    n = dims[0] * dims[1] * dims[2]
    if n != params.particleCount:
        raise ValueError(f"{path}: block holds {n} particles, ParticleCount is {params.particleCount}")
    pos = np.zeros((n, 4), np.float32)
    spacing = float(np.float32(params.h) * np.float32(params.setupSpacing))
    if lib().oracle_scene_block(dims[0], dims[1], dims[2], spacing, _ptr(origin), jitter, seed, _ptr(pos)) != 0:
        raise ValueError(f"{path}: no valid BlockDims")
    return params, pos, np.zeros_like(pos)


def set_wave_position(wave_pos: float = 0.0) -> None:
    """The moving wall (xMin + wave_pos) of every later oracle step."""
    lib().oracle_set_wave_position(float(wave_pos))


def render(cam, mode, params, pos):
    """The renderer's restatement: (splat, smooth, out) as [height, width, 4]
    float32 images (smooth is None outside mode 0).  cam: a ctypes PbfCamera."""
    n = int(params.particleCount)
    p = np.ascontiguousarray(pos, np.float32).reshape(n, 4)
    shape = (cam.height, cam.width, 4)
    splat, out = np.zeros(shape, np.float32), np.zeros(shape, np.float32)
    smooth = np.zeros(shape, np.float32) if mode == 0 else None
    rc = lib().oracle_render(ctypes.byref(cam), mode, n, float(params.h), _ptr(p), _ptr(splat), _ptr(smooth), _ptr(out))
    if rc != 0:
        raise ValueError("oracle_render rejected the arguments")
    return splat, smooth, out


def noise_sinf(x: float) -> float:
    return float(lib().oracle_noise_sinf(float(x)))


def _ptr(a):
    return None if a is None else a.ctypes.data


def n_keys(n: int) -> int:
    return (n + 2047) // 2048 * 2048


def step(params, pos, vel, substeps=1, paused=False, keys_state=None, threads=0, debug=False):
    """FP32 oracle.  Returns (pos, vel, pred[, debug dict])."""
    n = int(params.particleCount)
    pos = np.array(pos, np.float32, copy=True).reshape(n, 4)
    vel = np.array(vel, np.float32, copy=True).reshape(n, 4)
    pred = np.zeros((n, 4), np.float32)
    dbg = None
    out = {}
    if debug:
        slots = int(params.friendsCircles * params.particlesPerCircle)
        out = dict(keys=np.zeros(n_keys(n), np.uint32), perm=np.zeros(n_keys(n), np.uint32),
                   cells=np.zeros(2 * params.gridBufSize, np.uint32), counts=np.zeros((n, 2), np.uint32),
                   list=np.zeros((slots, n), np.uint32), density=np.zeros(n, np.float32),
                   lambda_=np.zeros(n, np.float32), omega=np.zeros((n, 4), np.float32))
        dbg = OracleDebug(_ptr(out["keys"]), _ptr(out["perm"]), _ptr(out["cells"]), _ptr(out["counts"]),
                          _ptr(out["list"]), slots, _ptr(out["density"]), _ptr(out["lambda_"]), _ptr(out["omega"]))
    rc = lib().oracle_step_f32(ctypes.byref(params), n, _ptr(pos), _ptr(vel), _ptr(pred), substeps, int(paused),
                               _ptr(keys_state), threads, ctypes.byref(dbg) if dbg is not None else None)
    if rc != 0:
        raise ValueError(f"oracle_step_f32 rejected the parameters ({rc})")
    return (pos, vel, pred, out) if debug else (pos, vel, pred)


def step_f64(params, pos, vel, substeps=1, threads=0):
    n = int(params.particleCount)
    pos = np.array(pos, np.float64, copy=True).reshape(n, 4)
    vel = np.array(vel, np.float64, copy=True).reshape(n, 4)
    pred = np.zeros((n, 4), np.float64)
    rc = lib().oracle_step_f64(ctypes.byref(params), n, _ptr(pos), _ptr(vel), _ptr(pred), substeps, threads)
    if rc != 0:
        raise ValueError(f"oracle_step_f64 rejected the parameters ({rc})")
    return pos, vel, pred


def sort(params, pred):
    n = int(params.particleCount)
    pred = np.ascontiguousarray(pred, np.float32).reshape(n, 4)
    keys = np.zeros(n_keys(n), np.uint32)
    perm = np.zeros(n_keys(n), np.uint32)
    cells = np.zeros(2 * params.gridBufSize, np.uint32)
    rc = lib().oracle_sort_f32(ctypes.byref(params), n, _ptr(pred), _ptr(keys), _ptr(perm), _ptr(cells))
    if rc != 0:
        raise ValueError(f"oracle_sort_f32 rejected the parameters ({rc})")
    return keys, perm, cells


def constants(params):
    a, b, c = c_float(), c_float(), c_float()
    lib().oracle_constants(ctypes.byref(params), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


def grid_hash(x, y, z, grid):
    return int(lib().oracle_grid_hash(x, y, z, grid))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def ref_max_threads() -> int:
    return int(ref().ref_max_threads())


def ref_step(params, pos, vel, substeps=1, threads=0):
    """The reference's kernels through the shim, work-items on `threads` host
    threads (0: all).  Returns (pos, vel, pred, keys, perm, cells)."""
    ref().ref_set_threads(int(threads))
    n = int(params.particleCount)
    pos = np.array(pos, np.float32, copy=True).reshape(n, 4)
    vel = np.array(vel, np.float32, copy=True).reshape(n, 4)
    pred = np.zeros((n, 4), np.float32)
    keys = np.zeros(n_keys(n), np.uint32)
    perm = np.zeros(n_keys(n), np.uint32)
    cells = np.zeros(2 * params.gridBufSize, np.uint32)
    rc = ref().ref_step_f32(ctypes.byref(params), n, _ptr(pos), _ptr(vel), _ptr(pred), substeps, _ptr(keys),
                            _ptr(perm), _ptr(cells))
    if rc != 0:
        raise ValueError(f"ref_step_f32 rejected the input ({rc})")
    return pos, vel, pred, keys, perm, cells


def ref_run_timed(params, pos, vel, warm, group, max_timed, budget_s, threads=0):
    """The reference's kernels through the shim: `warm` untimed substeps, then
    substeps timed in groups of `group` until `max_timed` have run or
    `budget_s` seconds have passed (buffer setup outside the clock).
    Returns (timed substeps, seconds, pos, vel)."""
    ref().ref_set_threads(int(threads))
    n = int(params.particleCount)
    pos = np.array(pos, np.float32, copy=True).reshape(n, 4)
    vel = np.array(vel, np.float32, copy=True).reshape(n, 4)
    done, secs = c_int(0), c_double(0.0)
    rc = ref().ref_run_timed(ctypes.byref(params), n, _ptr(pos), _ptr(vel), int(warm), int(group), int(max_timed),
                             float(budget_s), ctypes.byref(done), ctypes.byref(secs))
    if rc != 0:
        raise ValueError(f"ref_run_timed rejected the input ({rc})")
    return done.value, secs.value, pos, vel


def ref_sort(params, pred):
    n = int(params.particleCount)
    pred = np.ascontiguousarray(pred, np.float32).reshape(n, 4)
    keys = np.zeros(n_keys(n), np.uint32)
    perm = np.zeros(n_keys(n), np.uint32)
    cells = np.zeros(2 * params.gridBufSize, np.uint32)
    rc = ref().ref_sort_f32(ctypes.byref(params), n, _ptr(pred), _ptr(keys), _ptr(perm), _ptr(cells))
    if rc != 0:
        raise ValueError(f"ref_sort_f32 rejected the input ({rc})")
    return keys, perm, cells


class Rollout:
    """A rollout over a fixed neighbour structure: the FP32 forward (identical
    to the CUDA path) records the structure; replay() / grad() evaluate the
    same function with that structure frozen, in FP64."""

    def __init__(self, params, pos, vel, substeps, threads=0):
        n = int(params.particleCount)
        self.params = params
        self.n = n
        self.pos0 = np.array(pos, np.float32).reshape(n, 4)
        self.vel0 = np.array(vel, np.float32).reshape(n, 4)
        p = self.pos0.copy()
        v = self.vel0.copy()
        self.ids = np.zeros(n, np.uint32)
        self.handle = lib().oracle_rollout_record(ctypes.byref(params), n, _ptr(p), _ptr(v), substeps, _ptr(self.ids), threads)
        if not self.handle:
            raise ValueError("oracle_rollout_record rejected the input")
        self.pos_final32 = p  # final FP32 state, sorted order
        self.vel_final32 = v

    def __del__(self):
        if getattr(self, "handle", None):
            lib().oracle_rollout_free(self.handle)
            self.handle = None

    def final_by_id32(self):
        out = np.zeros_like(self.pos_final32)
        out[self.ids] = self.pos_final32
        return out

    def replay(self, vel0=None, gravity=None, visc=None, target=None):
        """(loss, final positions by id) in FP64; gravity (3) / visc override the recorded values."""
        v0 = np.ascontiguousarray(self.vel0 if vel0 is None else vel0, np.float64)
        p0 = np.ascontiguousarray(self.pos0, np.float64)
        out = np.zeros((self.n, 4), np.float64)
        tgt = None if target is None else np.ascontiguousarray(target, np.float64)
        g = None if gravity is None else np.ascontiguousarray(gravity, np.float64)
        vc = None if visc is None else c_double(visc)
        loss = lib().oracle_rollout_replay_f64(self.handle, _ptr(g), None if vc is None else ctypes.byref(vc),
                                               _ptr(p0), _ptr(v0), _ptr(tgt), _ptr(out))
        return loss, out

    def grad(self, target, vel0=None, gravity=None, visc=None):
        """(loss, dL/dv0 [n,4], dL/dviscosityFactor, dL/dgravity [3]) in FP64."""
        v0 = np.ascontiguousarray(self.vel0 if vel0 is None else vel0, np.float64)
        p0 = np.ascontiguousarray(self.pos0, np.float64)
        tgt = np.ascontiguousarray(target, np.float64)
        g = None if gravity is None else np.ascontiguousarray(gravity, np.float64)
        vc = None if visc is None else c_double(visc)
        dv = np.zeros((self.n, 4), np.float64)
        dc = c_double(0)
        dg = np.zeros(3, np.float64)
        loss = lib().oracle_rollout_grad_f64(self.handle, _ptr(g), None if vc is None else ctypes.byref(vc), _ptr(p0),
                                             _ptr(v0), _ptr(tgt), _ptr(dv), ctypes.byref(dc), _ptr(dg))
        return loss, dv, dc.value, dg

    def grad_f32(self, target, dl_dx=None):
        """The same reverse pass evaluated in FP32 (serial, fixed order):
        (loss, dL/dv0 [n,4], dL/dc, dL/dg [3]) as float64 arrays."""
        p0 = np.ascontiguousarray(self.pos0, np.float64)
        v0 = np.ascontiguousarray(self.vel0, np.float64)
        tgt = np.ascontiguousarray(target, np.float64)
        dx = None if dl_dx is None else np.ascontiguousarray(dl_dx, np.float64)
        dv = np.zeros((self.n, 4), np.float64)
        dc = c_double(0)
        dg = np.zeros(3, np.float64)
        loss = lib().oracle_rollout_grad_f32(self.handle, _ptr(p0), _ptr(v0), _ptr(tgt), _ptr(dx), _ptr(dv),
                                             ctypes.byref(dc), _ptr(dg))
        return loss, dv, dc.value, dg

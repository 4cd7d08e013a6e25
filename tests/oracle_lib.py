"""ctypes binding of the oracle (oracle/_build/liboracle.so) for the tests.

The oracle is the checker: a CPU restatement of the reference path tracer.
Only tests, the smoke check and the benchmark's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess
import threading

import numpy as np

from caustic import _abi

ROOT = pathlib.Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"
_lock = threading.Lock()
_lib = None
P = C.c_void_p


class or_camera_settings(C.Structure):
    _fields_ = [("target", C.c_double * 3), ("yaw", C.c_double), ("pitch", C.c_double),
                ("distance", C.c_double), ("fov_deg", C.c_double), ("lens_radius", C.c_double),
                ("focus_distance", C.c_double)]


def build() -> pathlib.Path:
    """Builds the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    return ORACLE_LIB


def lib() -> C.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(str(ORACLE_LIB))
            V = C.POINTER(_abi.ct_packed_scene_view)
            sig = {
                "or_pcg_hash": (C.c_uint32, [C.c_uint32]),
                "or_seed_for": (C.c_uint32, [C.c_uint32, C.c_uint32]),
                "or_rng_stream": (None, [C.c_uint32, C.c_uint32, C.c_int32, C.c_double, C.c_double, P]),
                "or_rng_stream_state": (C.c_uint32, [C.c_uint32, C.c_uint64, C.c_int32, C.c_double, C.c_double, P]),
                "or_pack": (P, [C.POINTER(_abi.ct_object), C.c_uint32, C.POINTER(_abi.ct_sky)]),
                "or_pack_cornell": (P, [C.POINTER(or_camera_settings)]),
                "or_packed_view": (None, [P, V, C.POINTER(C.POINTER(C.c_uint32))]),
                "or_packed_free": (None, [P]),
                "or_validate_bvh": (None, [V, P, C.c_uint32, P]),
                "or_trace": (None, [V, P, C.c_uint64, C.c_int32, P, P, P, P, P, C.c_int32]),
                "or_occluded": (None, [V, P, C.c_uint64, P, P, C.c_int32]),
                "or_prim_hit_t": (C.c_double, [V, C.c_int32, P]),
                "or_camera_frame": (None, [C.POINTER(or_camera_settings), C.c_double, C.POINTER(_abi.ct_camera_frame)]),
                "or_generate_ray": (None, [C.POINTER(_abi.ct_camera_frame), C.c_double, C.c_double, C.c_double,
                                           C.c_double, P]),
                "or_render_image": (None, [V, C.POINTER(_abi.ct_camera_frame), C.POINTER(_abi.ct_render_options),
                                           C.c_int32, P, P]),
                "or_accumulate_pass": (None, [V, C.POINTER(_abi.ct_camera_frame), C.c_int32, C.c_int32, C.c_uint32,
                                              C.POINTER(_abi.ct_trace_options), P, C.c_int32]),
                "or_pixel_radiance": (None, [V, C.POINTER(_abi.ct_camera_frame), C.c_int32, C.c_int32, C.c_uint32,
                                             C.c_uint32, C.POINTER(_abi.ct_trace_options), P, P]),
                "or_cornell_reference": (None, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]),
                "or_tonemap": (None, [P, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32, P]),
                "or_scalar": (C.c_double, [C.c_int32, C.c_double, C.c_double, C.c_double]),
                "or_vector": (None, [C.c_int32, P, P]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


def threads() -> int:
    return max(1, min(32, os.cpu_count() or 1))


class OraclePacked:
    """A scene packed by the oracle's restatement of packScene."""

    def __init__(self, handle):
        self.h = handle
        L = lib()
        self.view = _abi.ct_packed_scene_view()
        order = C.POINTER(C.c_uint32)()
        L.or_packed_view(self.h, C.byref(self.view), C.byref(order))
        v = self.view
        slots = max(1, v.prim_count)

        def arr(p, n, dt):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else np.zeros(0, dt)

        self.prims = arr(v.prims, slots * 16, np.float32)
        self.nodes = arr(v.nodes, v.node_count * 8, np.float32)
        self.mats = arr(v.mats, max(1, v.mat_count) * 16, np.float32)
        self.lights = arr(v.lights, v.light_count, np.int32)
        self.prim_object = arr(v.prim_object, slots, np.uint32)
        self.order = arr(order, v.prim_count, np.uint32)
        self.prim_count, self.node_count, self.mat_count = v.prim_count, v.node_count, v.mat_count

    def __del__(self):
        try:
            lib().or_packed_free(self.h)
        except Exception:
            pass


def pack(scene) -> OraclePacked:
    from caustic.pack import object_array, sky_struct

    arr, keep = object_array(scene.objects)
    sky = sky_struct(scene.sky)
    h = lib().or_pack(arr, len(scene.objects), C.byref(sky))
    out = OraclePacked(h)
    del keep
    return out


def pack_cornell():
    cam = or_camera_settings()
    return OraclePacked(lib().or_pack_cornell(C.byref(cam))), cam


def view_of(packed) -> _abi.ct_packed_scene_view:
    """ct_packed_scene_view of a caustic.PackedScene or an OraclePacked."""
    if isinstance(packed, OraclePacked):
        return packed.view
    return packed.view()


def validate(packed) -> dict:
    out = np.zeros(5, np.uint32)
    v = view_of(packed)
    lib().or_validate_bvh(C.byref(v), _p(packed.order), len(packed.order), _p(out))
    return dict(ok=bool(out[0]), max_leaf=int(out[1]), leaves=int(out[2]), depth=int(out[3]), errors=int(out[4]))


def trace(packed, rays: np.ndarray, mode: int = 0, nthreads: int | None = None):
    """mode 0 ordered walk, 1 stackless, 2 brute force -> (prim, t, u, v, counters)."""
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    n = len(rays)
    prim = np.empty(n, np.int32)
    t = np.empty(n, np.float64)
    u = np.empty(n, np.float64)
    v = np.empty(n, np.float64)
    cnt = np.zeros(4, np.uint64)
    view = view_of(packed)
    lib().or_trace(C.byref(view), _p(rays), n, mode, _p(prim), _p(t), _p(u), _p(v), _p(cnt),
                   nthreads or threads())
    return prim, t, u, v, cnt


def occluded(packed, rays: np.ndarray, nthreads: int | None = None):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    out = np.empty(len(rays), np.uint8)
    cnt = np.zeros(4, np.uint64)
    view = view_of(packed)
    lib().or_occluded(C.byref(view), _p(rays), len(rays), _p(out), _p(cnt), nthreads or threads())
    return out.astype(bool), cnt


def prim_hit_t(packed, prim: int, ray: np.ndarray) -> float:
    view = view_of(packed)
    r = np.ascontiguousarray(ray, np.float32)
    return lib().or_prim_hit_t(C.byref(view), int(prim), _p(r))


def rng_stream(seed: int, n: int, kind: int = 0, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().or_rng_stream(seed, n, kind, lo, hi, _p(out))
    return out


def rng_stream_state(state: int, out: np.ndarray, kind: int = 0, lo: float = 0.0, hi: float = 1.0) -> int:
    """Fills `out` (float64) with draws continuing from the raw xorshift `state`; returns the state reached.
    Same contract as caustic.rng's stream generators (installable with caustic.rng.set_stream)."""
    return int(lib().or_rng_stream_state(state, len(out), kind, lo, hi, _p(out)))


def camera_frame(settings: or_camera_settings, aspect: float) -> _abi.ct_camera_frame:
    f = _abi.ct_camera_frame()
    lib().or_camera_frame(C.byref(settings), aspect, C.byref(f))
    return f


def settings_struct(cam) -> or_camera_settings:
    s = or_camera_settings()
    s.target[:] = cam.target
    s.yaw, s.pitch, s.distance = cam.yaw, cam.pitch, cam.distance
    s.fov_deg, s.lens_radius, s.focus_distance = cam.fov_deg, cam.lens_radius, cam.focus_distance
    return s


def render_image(packed, frame: _abi.ct_camera_frame, opts: _abi.ct_render_options, nthreads: int | None = None,
                 want_sumsq: bool = False):
    out = np.empty(opts.width * opts.height * 3, np.float32)
    sumsq = np.zeros(opts.width * opts.height * 3, np.float64) if want_sumsq else None
    view = view_of(packed)
    lib().or_render_image(C.byref(view), C.byref(frame), C.byref(opts), nthreads or threads(), _p(out),
                          _p(sumsq))
    return (out, sumsq) if want_sumsq else out


def accumulate_pass(packed, frame, width, height, frame_index, topts, accum, nthreads: int | None = None):
    view = view_of(packed)
    lib().or_accumulate_pass(C.byref(view), C.byref(frame), width, height, frame_index, C.byref(topts),
                             _p(accum), nthreads or threads())


def pixel_radiance(packed, frame, width, height, pixel, frame_index, topts):
    """(radiance[3], work[10]) of one path; work as documented in oracle.h."""
    out = np.zeros(3, np.float64)
    work = np.zeros(10, np.uint64)
    view = view_of(packed)
    lib().or_pixel_radiance(C.byref(view), C.byref(frame), width, height, pixel, frame_index, C.byref(topts),
                            _p(out), _p(work))
    return out, work


def cornell_reference(width=96, height=64, spp=16, nthreads: int | None = None):
    linear = np.empty(width * height * 3, np.float32)
    rgba = np.empty(width * height * 4, np.uint8)
    lib().or_cornell_reference(width, height, spp, nthreads or threads(), _p(linear), _p(rgba))
    return linear, rgba


def tonemap(accum, width, height, samples, ev, aces=True):
    rgba = np.empty(width * height * 4, np.uint8)
    a = np.ascontiguousarray(accum, np.float32)
    lib().or_tonemap(_p(a), width, height, samples, ev, 1 if aces else 0, _p(rgba))
    return rgba


def scalar(fn: int, a: float, b: float = 0.0, c: float = 0.0) -> float:
    return lib().or_scalar(fn, a, b, c)


def vector(fn: int, args, nout: int = 6) -> np.ndarray:
    a = np.ascontiguousarray(args, np.float64)
    out = np.zeros(max(nout, 6), np.float64)
    lib().or_vector(fn, _p(a), _p(out))
    return out

"""GPU path tracer entry points (tracer.ts / intersect.ts surface).

`DeviceScene` owns a ct_scene: the packed arrays resident in HBM. The query
functions mirror intersectClosest/occluded over batches of rays; the render
functions mirror renderImage/accumulatePass. Every call goes through the CUDA
library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Union

import numpy as np

from . import _abi, _native
from .camera import CameraFrame
from .pack import PackedScene, pack_scene
from .scene import Scene

T_MIN = 1e-4  # intersect.ts:14


@dataclass(frozen=True)
class TraceOptions:
    """tracer.ts:27-33 (DEFAULT_TRACE_OPTIONS: 8 bounces, RR on, NEE on)."""

    max_bounces: int = 8
    russian_roulette: bool = True
    nee: bool = True

    def struct(self) -> _abi.ct_trace_options:
        return _abi.ct_trace_options(self.max_bounces, int(self.russian_roulette), int(self.nee))


@dataclass(frozen=True)
class RenderOptions(TraceOptions):
    """tracer.ts:337-342."""

    width: int = 0
    height: int = 0
    spp: int = 1
    seed: int = 0

    def struct(self) -> _abi.ct_render_options:
        return _abi.ct_render_options(self.width, self.height, self.spp, self.max_bounces,
                                      int(self.russian_roulette), int(self.nee), self.seed & 0xFFFFFFFF)


DEFAULT_TRACE_OPTIONS = TraceOptions()


class DeviceScene:
    """A PackedScene uploaded to the current CUDA device (ct_scene_create)."""

    def __init__(self, packed: PackedScene):
        self.packed = packed
        self._lib = _native.lib()
        handle = C.c_void_p()
        view = packed.view()
        _native.check(self._lib.ct_scene_create(C.byref(view), C.byref(handle)))
        self.handle = handle

    @classmethod
    def from_scene(cls, scene: Scene) -> "DeviceScene":
        return cls(pack_scene(scene))

    @property
    def device_bytes(self) -> int:
        return int(self._lib.ct_scene_device_bytes(self.handle))

    @property
    def walk(self) -> int:
        """Trace walk the integrator uses for this scene (0 ordered, 1 ordered
        with persistent refill, 2 stackless skip-link)."""
        return int(self._lib.ct_scene_walk(self.handle))

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._lib.ct_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def make_rays(origins: np.ndarray, dirs: np.ndarray, tmin: float = T_MIN,
              tmax: Union[float, np.ndarray] = np.inf) -> np.ndarray:
    """Packs rays into the (n, 8) float32 layout [ox oy oz dx dy dz tmin tmax]."""
    n = len(origins)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = origins
    rays[:, 3:6] = dirs
    rays[:, 6] = tmin
    rays[:, 7] = tmax
    return rays


@dataclass
class Hits:
    prim: np.ndarray  # int32, -1 = miss
    t: np.ndarray     # float32, inf = miss
    u: Optional[np.ndarray] = None
    v: Optional[np.ndarray] = None
    stats: Optional[_abi.ct_stats] = None


def intersect_closest(scene: DeviceScene, rays: np.ndarray, barycentrics: bool = False) -> Hits:
    """intersectClosest (intersect.ts:202-282) for each row of `rays` (n, 8) float32."""
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    n = len(rays)
    prim = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    u = np.empty(n, np.float32) if barycentrics else None
    v = np.empty(n, np.float32) if barycentrics else None
    stats = _abi.ct_stats()
    _native.check(scene._lib.ct_trace_closest(scene.handle, _native.ptr(rays), n, _native.ptr(prim),
                                              _native.ptr(t), _native.ptr(u), _native.ptr(v),
                                              C.byref(stats)))
    return Hits(prim, t, u, v, stats)


def occluded(scene: DeviceScene, rays: np.ndarray) -> np.ndarray:
    """occluded (intersect.ts:368-420) for each row of `rays`; returns bool array."""
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    out = np.empty(len(rays), np.uint8)
    _native.check(scene._lib.ct_trace_occluded(scene.handle, _native.ptr(rays), len(rays),
                                               _native.ptr(out), None))
    return out.astype(bool)


TRAVERSALS = {"ordered": 0, "stackless": 1, "ordered_thread": 2}


def set_traversal(variant: str) -> str:
    """Selects the query kernel: 'ordered' (short stack, persistent lanes),
    'stackless' (skip links) or 'ordered_thread' (short stack, one query per
    thread). Returns the previous variant."""
    prev = _native.lib().ct_set_traversal(TRAVERSALS[variant])
    return {v: k for k, v in TRAVERSALS.items()}[prev]


def accumulate_pass(scene: DeviceScene, frame: CameraFrame, width: int, height: int, frame_index: int,
                    opts: TraceOptions, accum: np.ndarray) -> None:
    """accumulatePass (tracer.ts:361-395): adds one sample per pixel into accum (float32, w*h*3)."""
    if accum.dtype != np.float32 or not accum.flags["C_CONTIGUOUS"] or accum.size != width * height * 3:
        raise ValueError("accum must be a contiguous float32 array of width*height*3 values")
    f = frame.struct()
    o = opts.struct() if type(opts) is TraceOptions else TraceOptions(
        opts.max_bounces, opts.russian_roulette, opts.nee).struct()
    _native.check(scene._lib.ct_accumulate_pass(scene.handle, C.byref(f), width, height, frame_index & 0xFFFFFFFF,
                                                C.byref(o), _native.ptr(accum), None))


def render_image(scene: Union[Scene, PackedScene, DeviceScene], frame: CameraFrame, opts: RenderOptions,
                 stats: Optional[_abi.ct_stats] = None) -> np.ndarray:
    """renderImage (tracer.ts:348-355): linear RGB float32 (h*w*3), row 0 = top, divided by spp."""
    own = None
    if isinstance(scene, Scene):
        scene = own = DeviceScene.from_scene(scene)
    elif isinstance(scene, PackedScene):
        scene = own = DeviceScene(scene)
    try:
        out = np.empty(opts.width * opts.height * 3, np.float32)
        o = opts.struct()
        f = frame.struct()
        _native.check(scene._lib.ct_render_image(scene.handle, C.byref(f), C.byref(o), _native.ptr(out),
                                                 C.byref(stats) if stats is not None else None))
        return out
    finally:
        if own is not None:
            own.close()


@dataclass
class PickResult:
    """picking.ts:7-12."""

    object_index: int
    prim: int
    t: float
    point: tuple


def pick_many(scene: DeviceScene, frame: CameraFrame, sx, sy):
    """pick (picking.ts:21-33) for arrays of screen positions on the GPU (ct_pick):
    returns (object, prim, t, point) arrays; object/prim -1 and t = inf on a miss."""
    sx = np.ascontiguousarray(sx, np.float64).reshape(-1)
    sy = np.ascontiguousarray(sy, np.float64).reshape(-1)
    n = len(sx)
    obj = np.empty(n, np.int32)
    prim = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    point = np.empty((n, 3), np.float64)
    f = frame.struct()
    _native.check(scene._lib.ct_pick(scene.handle, C.byref(f), n, _native.ptr(sx), _native.ptr(sy), _native.ptr(obj),
                                     _native.ptr(prim), _native.ptr(t), _native.ptr(point)))
    return obj, prim, t, point


def pick(scene: DeviceScene, frame: CameraFrame, sx: float, sy: float) -> Optional[PickResult]:
    """pick (picking.ts:21-33): what the pinhole ray through (sx, sy) hits, or None."""
    obj, prim, t, point = pick_many(scene, frame, [sx], [sy])
    if prim[0] < 0:
        return None
    return PickResult(int(obj[0]), int(prim[0]), float(t[0]), tuple(float(v) for v in point[0]))

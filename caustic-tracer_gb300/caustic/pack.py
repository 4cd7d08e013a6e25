"""packScene (pack.ts:195-223): Scene -> PackedScene float arrays.

The packing and binned-SAH BVH build run on the host in the library's C++
(ct_pack_scene); the arrays are bit-identical to the reference's
Float32Array/Int32Array/Uint32Array outputs.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _abi, _native
from .scene import (Dielectric, Emissive, Lambertian, Mesh, Metal, Quad, Scene, SceneObject, Sky,
                    SkyGradient, Sphere, Triangle)

PRIM_STRIDE = _abi.PRIM_STRIDE
NODE_STRIDE = _abi.NODE_STRIDE
MAT_STRIDE = _abi.MAT_STRIDE


@dataclass
class PackedScene:
    """PackedScene (pack.ts:46-59). Arrays are numpy; `order` maps packed slot -> scene-order primitive."""

    prims: np.ndarray        # float32 (max(1,prim_count) * 16)
    prim_count: int
    nodes: np.ndarray        # float32 (node_count * 8)
    node_count: int
    mats: np.ndarray         # float32 (max(1,mat_count) * 16)
    mat_count: int
    lights: np.ndarray       # int32
    prim_object: np.ndarray  # uint32
    sky: Sky
    order: np.ndarray        # uint32

    def view(self) -> _abi.ct_packed_scene_view:
        """ct_packed_scene_view borrowing this object's arrays (keep self alive while used)."""
        for name in ("prims", "nodes", "mats", "lights", "prim_object"):
            arr = getattr(self, name)
            if not arr.flags["C_CONTIGUOUS"]:
                setattr(self, name, np.ascontiguousarray(arr))
        v = _abi.ct_packed_scene_view()
        v.prims = self.prims.ctypes.data_as(C.POINTER(C.c_float))
        v.prim_count = self.prim_count
        v.nodes = self.nodes.ctypes.data_as(C.POINTER(C.c_float))
        v.node_count = self.node_count
        v.mats = self.mats.ctypes.data_as(C.POINTER(C.c_float))
        v.mat_count = self.mat_count
        v.lights = self.lights.ctypes.data_as(C.POINTER(C.c_int32))
        v.light_count = len(self.lights)
        v.prim_object = self.prim_object.ctypes.data_as(C.POINTER(C.c_uint32))
        v.sky = sky_struct(self.sky)
        return v

    @property
    def device_bytes_estimate(self) -> int:
        """Device bytes of the uploaded scene: the packed arrays, 64 B per
        interior node (4-wide records) and 96 B per primitive (plane records
        and the compact copy the exact tests read)."""
        interior = max(1, (self.node_count - 1) // 2)
        return (self.prims.nbytes + self.nodes.nbytes + self.mats.nbytes + self.lights.nbytes
                + self.prim_object.nbytes + 64 * interior + 96 * self.prim_count)


def sky_struct(sky: Sky) -> _abi.ct_sky:
    s = _abi.ct_sky()
    if isinstance(sky, SkyGradient):
        s.kind = 1
        s.zenith[:] = sky.zenith
        s.horizon[:] = sky.horizon
        s.strength = sky.strength
    return s


_MAT_CODE = {"lambertian": 0, "metal": 1, "dielectric": 2, "emissive": 3}


def _material(m, out: _abi.ct_material) -> None:
    out.type = _MAT_CODE[m.type]
    if isinstance(m, Lambertian):
        out.color[:] = m.albedo
        if m.checker is not None:
            out.has_checker = 1
            out.checker_color2[:] = m.checker.color2
            out.checker_scale = m.checker.scale
        if m.emission is not None:
            out.has_emission = 1
            out.emission[:] = m.emission
    elif isinstance(m, Metal):
        out.color[:] = m.albedo
        out.param = m.roughness
    elif isinstance(m, Dielectric):
        out.color[:] = m.tint if m.tint is not None else (1.0, 1.0, 1.0)
        out.param = m.ior
    elif isinstance(m, Emissive):
        out.color[:] = m.color
        out.param = m.strength
    else:
        raise TypeError(f"unknown material {m!r}")


def object_array(objects: Sequence[SceneObject]):
    """ct_object array for the scene's objects plus the numpy buffers it points into."""
    arr = (_abi.ct_object * max(1, len(objects)))()
    keep = []
    for i, obj in enumerate(objects):
        o = arr[i]
        sh = obj.shape
        if isinstance(sh, Sphere):
            o.shape.kind = 0
            o.shape.p[0:4] = [*sh.center, sh.radius]
        elif isinstance(sh, Triangle):
            o.shape.kind = 1
            o.shape.p[:] = [*sh.a, *sh.b, *sh.c]
        elif isinstance(sh, Quad):
            o.shape.kind = 2
            o.shape.p[:] = [*sh.origin, *sh.u, *sh.v]
        elif isinstance(sh, Mesh):
            verts = np.ascontiguousarray(sh.vertices, dtype=np.float64).reshape(-1)
            idx = np.ascontiguousarray(sh.indices, dtype=np.uint32).reshape(-1)
            keep += [verts, idx]
            o.shape.kind = 3
            o.shape.vertices = verts.ctypes.data_as(C.POINTER(C.c_double))
            o.shape.vertex_count = len(verts) // 3
            o.shape.indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
            o.shape.index_count = len(idx)
        else:
            raise TypeError(f"unknown shape {sh!r}")
        _material(obj.material, o.material)
    return arr, keep


def pack_scene(scene: Scene) -> PackedScene:
    """pack.ts:195-223."""
    lib = _native.lib()
    arr, keep = object_array(scene.objects)
    sky = sky_struct(scene.sky)
    out = C.POINTER(_abi.ct_packed_scene)()
    _native.check(lib.ct_pack_scene(arr, len(scene.objects), C.byref(sky), C.byref(out)))
    try:
        v = out.contents.view
        n_prim_slots = max(1, v.prim_count)

        def grab(p, n, dtype):
            if n == 0:
                return np.zeros(0, dtype)
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dtype, copy=True)

        packed = PackedScene(
            prims=grab(v.prims, n_prim_slots * PRIM_STRIDE, np.float32),
            prim_count=v.prim_count,
            nodes=grab(v.nodes, v.node_count * NODE_STRIDE, np.float32),
            node_count=v.node_count,
            mats=grab(v.mats, max(1, v.mat_count) * MAT_STRIDE, np.float32),
            mat_count=v.mat_count,
            lights=grab(v.lights, v.light_count, np.int32),
            prim_object=grab(v.prim_object, n_prim_slots, np.uint32),
            sky=scene.sky,
            order=grab(out.contents.order, v.prim_count, np.uint32),
        )
    finally:
        lib.ct_packed_scene_free(out)
    del keep
    return packed

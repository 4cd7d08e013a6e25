"""Scene model (scene.ts:21-74): shapes, materials, sky, camera settings.

Vectors and colours are plain (x, y, z) / (r, g, b) tuples of floats; meshes
hold numpy arrays so million-triangle soups stay compact.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence, Tuple, Union

import numpy as np

Vec3 = Tuple[float, float, float]
Color = Tuple[float, float, float]


# ---- materials (scene.ts:21-31) ------------------------------------------------
@dataclass(frozen=True)
class CheckerTexture:
    color2: Color
    scale: float


@dataclass(frozen=True)
class Lambertian:
    albedo: Color
    checker: Optional[CheckerTexture] = None
    emission: Optional[Color] = None
    type: str = "lambertian"


@dataclass(frozen=True)
class Metal:
    albedo: Color
    roughness: float
    type: str = "metal"


@dataclass(frozen=True)
class Dielectric:
    ior: float
    tint: Optional[Color] = None
    type: str = "dielectric"


@dataclass(frozen=True)
class Emissive:
    color: Color
    strength: float
    type: str = "emissive"


Material = Union[Lambertian, Metal, Dielectric, Emissive]


# ---- shapes (scene.ts:35-41) ---------------------------------------------------
@dataclass(frozen=True)
class Sphere:
    center: Vec3
    radius: float
    kind: str = "sphere"


@dataclass(frozen=True)
class Triangle:
    a: Vec3
    b: Vec3
    c: Vec3
    kind: str = "triangle"


@dataclass(frozen=True)
class Quad:
    """Parallelogram spanned by u and v from origin; two triangles."""

    origin: Vec3
    u: Vec3
    v: Vec3
    kind: str = "quad"


@dataclass(frozen=True, eq=False)
class Mesh:
    """Indexed triangle mesh: vertices (N, 3) float64, indices (3M,) uint32."""

    vertices: np.ndarray
    indices: np.ndarray
    kind: str = "mesh"


Shape = Union[Sphere, Triangle, Quad, Mesh]


@dataclass(frozen=True)
class SceneObject:
    id: str
    name: str
    shape: Shape
    material: Material


# ---- sky and camera (scene.ts:50-67) ------------------------------------------
@dataclass(frozen=True)
class SkyNone:
    kind: str = "none"


@dataclass(frozen=True)
class SkyGradient:
    zenith: Color
    horizon: Color
    strength: float
    kind: str = "gradient"


Sky = Union[SkyNone, SkyGradient]


@dataclass(frozen=True)
class CameraSettings:
    target: Vec3
    yaw: float
    pitch: float
    distance: float
    fov_deg: float
    lens_radius: float
    focus_distance: float


@dataclass(frozen=True)
class Scene:
    name: str
    objects: Sequence[SceneObject]
    camera: CameraSettings
    sky: Sky = field(default_factory=SkyNone)


# ---- helpers (scene.ts:85-185) -----------------------------------------------------
def _add(a: Vec3, b: Vec3) -> Vec3:
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def _sub(a: Vec3, b: Vec3) -> Vec3:
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _cross(a: Vec3, b: Vec3) -> Vec3:
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def quad_triangles(origin: Vec3, u: Vec3, v: Vec3):
    """scene.ts:85-94."""
    p0 = origin
    p1 = _add(origin, u)
    p2 = _add(_add(origin, u), v)
    p3 = _add(origin, v)
    return [(p0, p1, p2), (p0, p2, p3)]


def triangle_normal(a: Vec3, b: Vec3, c: Vec3) -> Vec3:
    """scene.ts:120-122."""
    n = _cross(_sub(b, a), _sub(c, a))
    length = math.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
    if length > 0:
        inv = 1 / length
        return (n[0] * inv, n[1] * inv, n[2] * inv)
    return (0.0, 0.0, 0.0)


def triangle_area(a: Vec3, b: Vec3, c: Vec3) -> float:
    """scene.ts:124-127."""
    n = _cross(_sub(b, a), _sub(c, a))
    return 0.5 * math.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])


def primitive_count(shape: Shape) -> int:
    """scene.ts:129-140."""
    if isinstance(shape, (Sphere, Triangle)):
        return 1
    if isinstance(shape, Quad):
        return 2
    return int(len(shape.indices) // 3)


def material_emission(m: Material) -> Optional[Color]:
    """scene.ts:176-185: emitted radiance, or None for non-emitters."""
    if isinstance(m, Emissive):
        return (m.color[0] * m.strength, m.color[1] * m.strength, m.color[2] * m.strength)
    if isinstance(m, Lambertian) and m.emission is not None:
        e = m.emission
        if e[0] > 0 or e[1] > 0 or e[2] > 0:
            return e
    return None

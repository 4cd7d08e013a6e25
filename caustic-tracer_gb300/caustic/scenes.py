"""Scenes: the reference's Cornell preset and the synthetic workloads.

* CORNELL_BOX, cornell_box(): scenes.ts:45-67 (the reference's preset).
* furnace_scene(): furnace.test.ts:13-25 (closed emissive-diffuse sphere).
* random_test_scene(): bvh.test.ts:9-43 (spheres + triangles from Rng).
* cornell_unit_box(): Cornell box of the benchmark (unit room, 10 wall
  triangles, 0.25 x 0.25 light of emission 15, metal and glass spheres r 0.18).
* triangle_soup() / soup_rays(): traversal workload (1,000,000 triangles with
  centroids uniform in [-0.5,0.5]^3 and vertex offsets in +-0.01; rays from a
  radius-2 sphere towards uniform points of the cube).
* caustic_scene(): level-7 icosphere (327,680 triangles) displaced by value
  noise, 64 spheres, checker ground, small spherical emitter.
All random choices come from the reference's Rng with fixed seeds.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from .camera import camera_at
from .rng import Rng
from .scene import (CameraSettings, CheckerTexture, Dielectric, Emissive, Lambertian, Mesh, Metal,
                    Quad, Scene, SceneObject, SkyNone, Sphere, Triangle)


def _obj(name: str, shape, material, idx: List[int]) -> SceneObject:
    idx[0] += 1
    return SceneObject(id=f"p{idx[0]:x}", name=name, shape=shape, material=material)


def cornell_box() -> Scene:
    """The reference's CORNELL_BOX preset (scenes.ts:45-67): 1.5 x 1 x 1 room."""
    white = Lambertian((0.73, 0.73, 0.73))
    red = Lambertian((0.65, 0.05, 0.05))
    green = Lambertian((0.12, 0.45, 0.15))
    W = 0.75
    n = [0]
    objects = [
        _obj("Floor", Quad((-W, 0, -0.5), (2 * W, 0, 0), (0, 0, 1)), white, n),
        _obj("Ceiling", Quad((-W, 1, -0.5), (2 * W, 0, 0), (0, 0, 1)), white, n),
        _obj("Back wall", Quad((-W, 0, -0.5), (2 * W, 0, 0), (0, 1, 0)), white, n),
        _obj("Red wall", Quad((-W, 0, -0.5), (0, 0, 1), (0, 1, 0)), red, n),
        _obj("Green wall", Quad((W, 0, -0.5), (0, 0, 1), (0, 1, 0)), green, n),
        _obj("Ceiling light", Quad((-0.2, 0.998, -0.15), (0.4, 0, 0), (0, 0, 0.3)),
             Emissive((1, 0.86, 0.7), 12), n),
        _obj("Metal sphere", Sphere((-0.33, 0.24, -0.12), 0.24), Metal((0.9, 0.9, 0.92), 0.02), n),
        _obj("Glass sphere", Sphere((0.3, 0.2, 0.17), 0.2), Dielectric(1.5), n),
    ]
    return Scene("Cornell Box", objects, camera_at((0, 0.5, 1.6), (0, 0.5, 0), 32, 0, 1.6), SkyNone())


CORNELL_BOX = cornell_box()


def furnace_scene() -> Scene:
    """furnace.test.ts:13-25: camera inside a radius-5 sphere, albedo 0.8, emission 1."""
    shell = SceneObject("shell", "shell", Sphere((0, 0, 0), 5),
                        Lambertian((0.8, 0.8, 0.8), emission=(1, 1, 1)))
    cam = CameraSettings(target=(0, 0, -1), yaw=0, pitch=0, distance=1, fov_deg=60, lens_radius=0, focus_distance=1)
    return Scene("furnace", [shell], cam, SkyNone())


def random_test_scene(rng: Rng, spheres: int, triangles: int) -> Scene:
    """bvh.test.ts:9-43 (draw order: sphere centre xyz, radius; triangle a xyz, b offsets, c offsets)."""
    grey = Lambertian((0.5, 0.5, 0.5))
    objects = []
    for i in range(spheres):
        c = (rng.range(-10, 10), rng.range(-10, 10), rng.range(-10, 10))
        objects.append(SceneObject(f"s{i}", f"s{i}", Sphere(c, rng.range(0.05, 0.6)), grey))
    for i in range(triangles):
        a = (rng.range(-10, 10), rng.range(-10, 10), rng.range(-10, 10))
        b = (a[0] + rng.range(-1, 1), a[1] + rng.range(-1, 1), a[2] + rng.range(-1, 1))
        c = (a[0] + rng.range(-1, 1), a[1] + rng.range(-1, 1), a[2] + rng.range(-1, 1))
        objects.append(SceneObject(f"t{i}", f"t{i}", Triangle(a, b, c), grey))
    cam = CameraSettings(target=(0, 0, 0), yaw=0, pitch=0, distance=30, fov_deg=40, lens_radius=0, focus_distance=30)
    return Scene("random", objects, cam, SkyNone())


def cornell_unit_box() -> Scene:
    """Cornell box of the benchmark configuration.

    Unit room x in [-0.5, 0.5], y in [0, 1], z in [-0.5, 0.5]: floor, ceiling
    and back wall white 0.73, left wall red (0.65, 0.05, 0.05), right wall green
    (0.12, 0.45, 0.15) -> 10 triangles; a 0.25 x 0.25 ceiling light quad at
    y = 0.998 with emission 15 (2 triangles); a metal sphere (fuzz 0, albedo
    0.9/0.9/0.92) and a glass sphere (IOR 1.5), both radius 0.18 on the floor.
    Camera as the reference's Cornell preset (eye (0, 0.5, 1.6), 32 degrees).
    """
    white = Lambertian((0.73, 0.73, 0.73))
    n = [0]
    objects = [
        _obj("Floor", Quad((-0.5, 0, -0.5), (1, 0, 0), (0, 0, 1)), white, n),
        _obj("Ceiling", Quad((-0.5, 1, -0.5), (1, 0, 0), (0, 0, 1)), white, n),
        _obj("Back wall", Quad((-0.5, 0, -0.5), (1, 0, 0), (0, 1, 0)), white, n),
        _obj("Red wall", Quad((-0.5, 0, -0.5), (0, 0, 1), (0, 1, 0)), Lambertian((0.65, 0.05, 0.05)), n),
        _obj("Green wall", Quad((0.5, 0, -0.5), (0, 0, 1), (0, 1, 0)), Lambertian((0.12, 0.45, 0.15)), n),
        _obj("Ceiling light", Quad((-0.125, 0.998, -0.125), (0.25, 0, 0), (0, 0, 0.25)), Emissive((1, 1, 1), 15), n),
        _obj("Metal sphere", Sphere((-0.22, 0.18, -0.15), 0.18), Metal((0.9, 0.9, 0.92), 0.0), n),
        _obj("Glass sphere", Sphere((0.22, 0.18, 0.1), 0.18), Dielectric(1.5), n),
    ]
    return Scene("Cornell unit box", objects, camera_at((0, 0.5, 1.6), (0, 0.5, 0), 32, 0, 1.6), SkyNone())


def triangle_soup(count: int = 1_000_000, seed: int = 2024, half: float = 0.5, jitter: float = 0.01) -> Scene:
    """`count` triangles: centroid c ~ U(-half, half)^3, vertices c + U(-jitter, jitter)^3.

    Draw order per triangle: cx, cy, cz, then a, b, c offsets (x, y, z each),
    all from one Rng(seed) stream. One mesh object, grey Lambertian.
    """
    u = Rng(seed).draw(count * 12).reshape(count, 12)
    centre = -half + (half - -half) * u[:, 0:3]
    offs = -jitter + (jitter - -jitter) * u[:, 3:12]
    verts = (np.repeat(centre, 3, axis=0) + offs.reshape(count * 3, 3)).astype(np.float64)
    idx = np.arange(count * 3, dtype=np.uint32)
    mesh = Mesh(verts, idx)
    cam = camera_at((0, 0, 2.2), (0, 0, 0), 40, 0)
    return Scene("triangle soup", [SceneObject("soup", "soup", mesh, Lambertian((0.5, 0.5, 0.5)))], cam, SkyNone())


def soup_rays(count: int, seed: int = 77, radius: float = 2.0, half: float = 0.5) -> np.ndarray:
    """Rays (count, 8) float32: origin = radius * unitVector(u1, u2) (materials.ts:67-74),
    direction = normalize(target - origin), target ~ U(-half, half)^3, tmin 1e-4, tmax inf."""
    u = Rng(seed).draw(count * 5).reshape(count, 5)
    z = 1 - 2 * u[:, 0]
    r = np.sqrt(np.where(z * z < 1, 1 - z * z, 0.0))
    phi = (2 * math.pi) * u[:, 1]
    origin = radius * np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    target = -half + (half - -half) * u[:, 2:5]
    d = target - origin
    d /= np.sqrt((d * d).sum(axis=1, keepdims=True))
    rays = np.empty((count, 8), np.float32)
    rays[:, 0:3] = origin
    rays[:, 3:6] = d
    rays[:, 6] = 1e-4
    rays[:, 7] = np.inf
    return rays


# ---- caustic scene ---------------------------------------------------------------

def icosphere(level: int) -> Tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: 20 * 4**level faces, vertices on the unit sphere."""
    t = (1 + math.sqrt(5)) / 2
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
                  (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
                  (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
                  (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * len(v) + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // len(v), uniq % len(v)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + len(v)  # midpoint of edges (01, 12, 20) per face
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m[0], m[2]], 1), np.stack([f[:, 1], m[1], m[0]], 1),
            np.stack([f[:, 2], m[2], m[1]], 1), np.stack([m[0], m[1], m[2]], 1)])
    return v, f


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3D value noise in [-1, 1]: lattice values from pcg_hash, smoothstep trilinear blend."""
    cell = np.floor(p)
    frac = p - cell
    w = frac * frac * (3 - 2 * frac)
    ci = cell.astype(np.int64)

    def lattice(ix, iy, iz):
        h = (ix * 73856093 ^ iy * 19349663 ^ iz * 83492791 ^ seed) & 0xFFFFFFFF
        return _pcg_vec(h).astype(np.float64) / 4294967295.0 * 2 - 1

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out = out + wx * wy * wz * lattice(ci[:, 0] + dx, ci[:, 1] + dy, ci[:, 2] + dz)
    return out


def _pcg_vec(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64) & 0xFFFFFFFF
    state = (x * 747796405 + 2891336453) & 0xFFFFFFFF
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((word >> 22) ^ word) & 0xFFFFFFFF


def _random_material(rng: Rng):
    pick = rng.next()
    if pick < 0.4:
        return Lambertian((rng.range(0.1, 0.9), rng.range(0.1, 0.9), rng.range(0.1, 0.9)))
    if pick < 0.7:
        return Metal((rng.range(0.5, 1.0), rng.range(0.5, 1.0), rng.range(0.5, 1.0)), rng.range(0.0, 0.3))
    return Dielectric(1.5)


def batch_scene(seed: int, triangles: int, spheres: int) -> Scene:
    """One scene of the batched workload: a triangle soup as in triangle_soup()
    (Lambertian, random albedo), `spheres` spheres of radius U(0.02, 0.08)
    inside the cube with materials drawn as in caustic_scene(), and one
    0.3 x 0.3 ceiling light quad above the cube with emission 15."""
    rng = Rng(seed)
    soup = triangle_soup(triangles, seed=seed * 7 + 1)
    n = [0]
    albedo = (rng.range(0.2, 0.9), rng.range(0.2, 0.9), rng.range(0.2, 0.9))
    objects = [SceneObject("soup", "soup", soup.objects[0].shape, Lambertian(albedo)),
               _obj("Light", Quad((-0.15, 0.7, -0.15), (0.3, 0, 0), (0, 0, 0.3)), Emissive((1, 1, 1), 15), n)]
    for i in range(spheres):
        c = (rng.range(-0.45, 0.45), rng.range(-0.45, 0.45), rng.range(-0.45, 0.45))
        objects.append(_obj(f"Sphere {i + 1}", Sphere(c, rng.range(0.02, 0.08)), _random_material(rng), n))
    return Scene(f"batch {seed}", objects, camera_at((0.0, 0.3, 2.0), (0, 0, 0), 45, 0), SkyNone())


def batch_workload(count: int = 256, seed: int = 4096, min_tris: int = 2_000, max_tris: int = 200_000,
                   max_spheres: int = 32, sizes=(64, 128, 256, 512)):
    """(scene, width, height) for `count` batched-workload scenes: triangle counts
    log-uniform in [min_tris, max_tris], 0..max_spheres spheres, square images
    with a side drawn uniformly from `sizes` (all choices from Rng(seed))."""
    rng = Rng(seed)
    out = []
    lo, hi = math.log(min_tris), math.log(max_tris)
    for i in range(count):
        tris = int(round(math.exp(rng.range(lo, hi))))
        spheres = rng.int(max_spheres + 1)
        side = sizes[rng.int(len(sizes))]
        out.append((batch_scene(seed + 1 + i, tris, spheres), side, side))
    return out


def caustic_scene(seed: int = 7, level: int = 7) -> Scene:
    """Caustic workload: glass icosphere (level 7 = 327,680 triangles, radius 0.8,
    radial value-noise displacement of amplitude 0.05), 64 spheres of radius
    U(0.05, 0.2) with materials 40% Lambertian / 30% metal (fuzz U(0, 0.3)) /
    30% glass (IOR 1.5), a 2-triangle checker ground and one spherical emitter
    of radius 0.1 and emission 50."""
    rng = Rng(seed)
    v, f = icosphere(level)
    disp = 0.8 + 0.05 * value_noise(v * 3.0, seed)
    verts = v * disp[:, None] + np.array([0.0, 1.0, 0.0])
    n = [0]
    objects = [
        _obj("Checker ground", Quad((-20, 0, -20), (40, 0, 0), (0, 0, 40)),
             Lambertian((0.8, 0.8, 0.8), CheckerTexture((0.2, 0.2, 0.2), 2.0)), n),
        _obj("Glass blob", Mesh(verts, f.reshape(-1).astype(np.uint32)), Dielectric(1.5), n),
    ]
    for i in range(64):
        r = rng.range(0.05, 0.2)
        ang = rng.range(0, 2 * math.pi)
        dist = rng.range(1.1, 3.0)
        c = (dist * math.cos(ang), r, dist * math.sin(ang))
        objects.append(_obj(f"Sphere {i + 1}", Sphere(c, r), _random_material(rng), n))
    objects.append(_obj("Light", Sphere((1.5, 3.0, 1.0), 0.1), Emissive((1, 1, 1), 50), n))
    return Scene("caustic", objects, camera_at((0, 1.6, 4.5), (0, 0.7, 0), 40, 0), SkyNone())

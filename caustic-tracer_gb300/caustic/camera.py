"""Thin-lens camera (camera.ts): orbit settings -> world-space CameraFrame."""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

from . import _abi
from .scene import CameraSettings, Vec3


@dataclass(frozen=True)
class CameraFrame:
    """camera.ts:8-20."""

    origin: Vec3
    right: Vec3
    up: Vec3
    forward: Vec3
    tan_half_fov: float
    aspect: float
    lens_radius: float
    focus_distance: float

    def struct(self) -> _abi.ct_camera_frame:
        f = _abi.ct_camera_frame()
        f.origin[:] = self.origin
        f.right[:] = self.right
        f.up[:] = self.up
        f.forward[:] = self.forward
        f.tan_half_fov = self.tan_half_fov
        f.aspect = self.aspect
        f.lens_radius = self.lens_radius
        f.focus_distance = self.focus_distance
        return f


def _normalize(a: Vec3) -> Vec3:
    length = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
    if length > 0:
        s = 1 / length
        return (a[0] * s, a[1] * s, a[2] * s)
    return (0.0, 0.0, 0.0)


def _cross(a: Vec3, b: Vec3) -> Vec3:
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def camera_position(cam: CameraSettings) -> Vec3:
    """camera.ts:25-31."""
    cp = math.cos(cam.pitch)
    d = cam.distance
    return (cam.target[0] + (cp * math.sin(cam.yaw)) * d,
            cam.target[1] + math.sin(cam.pitch) * d,
            cam.target[2] + (cp * math.cos(cam.yaw)) * d)


def camera_frame(cam: CameraSettings, aspect: float) -> CameraFrame:
    """camera.ts:33-51."""
    origin = camera_position(cam)
    forward = _normalize((cam.target[0] - origin[0], cam.target[1] - origin[1], cam.target[2] - origin[2]))
    right = _cross(forward, (0.0, 1.0, 0.0))
    if right[0] * right[0] + right[1] * right[1] + right[2] * right[2] < 1e-12:
        right = (1.0, 0.0, 0.0)
    right = _normalize(right)
    up = _cross(right, forward)
    return CameraFrame(origin, right, up, forward, math.tan((cam.fov_deg * math.pi) / 360), aspect,
                       cam.lens_radius, max(1e-3, cam.focus_distance))


def camera_at(eye: Vec3, target: Vec3, fov_deg: float, lens_radius: float,
              focus_distance: Optional[float] = None) -> CameraSettings:
    """Orbit camera at `eye` looking at `target` (scenes.ts:26-40)."""
    dx, dy, dz = eye[0] - target[0], eye[1] - target[1], eye[2] - target[2]
    distance = math.sqrt(dx * dx + dy * dy + dz * dz)
    return CameraSettings(target=target, yaw=math.atan2(dx, dz), pitch=math.asin(dy / distance),
                          distance=distance, fov_deg=fov_deg, lens_radius=lens_radius,
                          focus_distance=distance if focus_distance is None else focus_distance)


def generate_ray(f: CameraFrame, sx: float, sy: float, lens_x: float, lens_y: float):
    """camera.ts:62-72: (origin, unit direction) through screen point (sx, sy), y up."""
    px = (2 * sx - 1) * f.tan_half_fov * f.aspect
    py = (2 * sy - 1) * f.tan_half_fov
    focus = tuple(f.origin[k] + ((f.right[k] * px + f.up[k] * py) + f.forward[k]) * f.focus_distance
                  for k in range(3))
    origin = tuple(f.origin[k] + (f.right[k] * (lens_x * f.lens_radius) + f.up[k] * (lens_y * f.lens_radius))
                   for k in range(3))
    return origin, _normalize(tuple(focus[k] - origin[k] for k in range(3)))

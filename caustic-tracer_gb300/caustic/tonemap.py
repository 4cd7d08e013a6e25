"""Display transforms (tonemap.ts) and binary PPM (ppm.ts), on the host."""
from __future__ import annotations

import math

import numpy as np


def aces_fitted(x):
    """tonemap.ts:7-15 (vectorised)."""
    x = np.asarray(x, np.float64)
    v = (x * (2.51 * x + 0.03)) / (x * (2.43 * x + 0.59) + 0.14)
    return np.clip(v, 0.0, 1.0)


def reinhard(x):
    """tonemap.ts:18-20."""
    x = np.asarray(x, np.float64)
    return np.where(x <= 0, 0.0, x / (1 + np.maximum(x, 0)))


def linear_to_srgb(x):
    """tonemap.ts:27-31."""
    x = np.asarray(x, np.float64)
    lo = 12.92 * x
    hi = 1.055 * np.power(np.clip(x, 0.0031308, 1.0), 1 / 2.4) - 0.055
    out = np.where(x <= 0.0031308, lo, hi)
    return np.where(x <= 0, 0.0, np.where(x >= 1, 1.0, out))


def js_round(x):
    """JavaScript Math.round: nearest integer, halves toward +infinity."""
    x = np.asarray(x, np.float64)
    f = np.floor(x)
    return np.where(x - f >= 0.5, f + 1, f)


def tonemap_buffer(accum: np.ndarray, width: int, height: int, samples: float, exposure_ev: float = 0.0,
                   mode: str = "aces") -> np.ndarray:
    """tonemap.ts:41-62: accumulated linear RGB (sum over samples) -> uint8 RGBA."""
    inv = math.pow(2.0, exposure_ev) / samples if samples > 0 else 0.0
    rgb = np.asarray(accum, np.float32).reshape(height * width, 3).astype(np.float64) * inv
    mapped = aces_fitted(rgb) if mode == "aces" else reinhard(rgb)
    q = np.clip(js_round(linear_to_srgb(mapped) * 255), 0, 255).astype(np.uint8)
    rgba = np.full((height * width, 4), 255, np.uint8)
    rgba[:, :3] = q
    return rgba.reshape(-1)


def encode_ppm(width: int, height: int, rgba: np.ndarray) -> bytes:
    """ppm.ts:4-16."""
    px = np.asarray(rgba, np.uint8).reshape(width * height, 4)[:, :3]
    return f"P6\n{width} {height}\n255\n".encode() + px.tobytes()


def decode_ppm(data: bytes):
    """ppm.ts:25-47: returns (width, height, rgb uint8 (h*w*3))."""
    tokens, i = [], 0
    while len(tokens) < 4 and i < len(data):
        while i < len(data) and data[i] in b" \n\r\t":
            i += 1
        if data[i:i + 1] == b"#":
            while i < len(data) and data[i] != 0x0A:
                i += 1
            continue
        start = i
        while i < len(data) and data[i] not in b" \n\r\t":
            i += 1
        tokens.append(data[start:i].decode())
    if tokens[0] != "P6":
        raise ValueError("not a binary PPM")
    if tokens[3] != "255":
        raise ValueError("only maxval 255 supported")
    w, h = int(tokens[1]), int(tokens[2])
    i += 1
    rgb = np.frombuffer(data[i:i + w * h * 3], np.uint8)
    if len(rgb) != w * h * 3:
        raise ValueError("truncated PPM data")
    return w, h, rgb

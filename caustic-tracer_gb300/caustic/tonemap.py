"""Display transforms (tonemap.ts) and binary PPM (ppm.ts).

`tonemap_device` / `ppm_device` run the transform on the GPU
(ct_tonemap_device / ct_ppm_device) on a device sum buffer; the numpy forms
below serve host arrays (the reference's own helpers run on the host too).
"""
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


MODES = {"aces": 0, "reinhard": 1}


def tonemap_device(accum, width: int, height: int, samples: float, exposure_ev: float = 0.0, mode: str = "aces",
                   stream=None):
    """tonemapBuffer on the GPU: `accum` is a CUDA float32 tensor of width*height*3
    sums; returns a CUDA uint8 tensor of width*height*4 RGBA bytes (equal to
    tonemap_buffer's)."""
    import ctypes as C

    import torch

    from . import _native

    lib = _native.lib()
    out = torch.empty(width * height * 4, dtype=torch.uint8, device=accum.device)
    s = C.c_void_p(stream.cuda_stream) if stream is not None else C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _native.check(lib.ct_tonemap_device(C.c_void_p(accum.data_ptr()), width, height, float(samples),
                                        float(exposure_ev), MODES[mode], C.c_void_p(out.data_ptr()), s))
    return out


def ppm_device(accum, width: int, height: int, samples: float, exposure_ev: float = 0.0, mode: str = "aces",
               stream=None) -> bytes:
    """tonemapBuffer + encodePPM on the GPU; returns the PPM file bytes."""
    import ctypes as C

    import torch

    from . import _native

    lib = _native.lib()
    cap = 32 + width * height * 3
    out = torch.empty(cap, dtype=torch.uint8, device=accum.device)
    size = C.c_uint64()
    s = C.c_void_p(stream.cuda_stream) if stream is not None else C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _native.check(lib.ct_ppm_device(C.c_void_p(accum.data_ptr()), width, height, float(samples), float(exposure_ev),
                                    MODES[mode], C.c_void_p(out.data_ptr()), cap, C.byref(size), s))
    return out[:size.value].cpu().numpy().tobytes()

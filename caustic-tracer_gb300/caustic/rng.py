"""Deterministic 32-bit RNG of the reference (rng.ts:10-65).

`Rng` is the scalar form for small scene generators; `Rng.draw(n)` produces
long streams through the library's ct_rng_stream so generators of million-
triangle scenes stay fast while consuming the identical sequence. A process
that must not load the CUDA library (a CPU-only tool timing another
implementation on the same inputs) installs another generator of the same
stream with `set_stream`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

M32 = 0xFFFFFFFF

# stream(state, out, kind, lo, hi) -> new state; None = the library's ct_rng_stream
_stream = None


def set_stream(fn):
    """Installs the generator behind Rng.draw and returns the previous one.

    fn(state, out, kind, lo, hi) fills the float64 array `out` with draws
    continuing from the raw xorshift `state` (kind 0 next(), 1 nextU32(),
    2 range(lo, hi)) and returns the state reached. None restores the
    library's ct_rng_stream."""
    global _stream
    prev, _stream = _stream, fn
    return prev


def pcg_hash(x: int) -> int:
    """rng.ts:10-15."""
    state = (x * 747796405 + 2891336453) & M32
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & M32
    return ((word >> 22) ^ word) & M32


def seed_for(pixel_index: int, frame: int) -> int:
    """rng.ts:18-23."""
    a = pcg_hash(pixel_index & M32)
    b = pcg_hash((frame & M32) ^ 0x9E3779B9)
    s = pcg_hash((a ^ ((b * 0x85EBCA6B) & M32)) & M32)
    return 0x1234567 if s == 0 else s


class Rng:
    """xorshift32 stream seeded through pcg_hash (rng.ts:25-65)."""

    def __init__(self, seed: int):
        s = pcg_hash(int(seed) & M32)
        self.state = 0x9E3779B9 if s == 0 else s

    @staticmethod
    def from_pixel(pixel_index: int, frame: int) -> "Rng":
        r = Rng(0)
        r.state = seed_for(pixel_index, frame)
        return r

    def next_u32(self) -> int:
        x = self.state
        x ^= (x << 13) & M32
        x ^= x >> 17
        x ^= (x << 5) & M32
        self.state = x
        return x

    def next(self) -> float:
        return self.next_u32() / 4294967296.0

    def range(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.next()

    def int(self, n: int) -> int:
        import math

        return min(n - 1, math.floor(self.next() * n))

    def draw(self, n: int, kind: str = "next", lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """n consecutive draws (kind 'next', 'u32' or 'range'), advancing this stream."""
        out = np.empty(int(n), np.float64)
        k = {"next": 0, "u32": 1, "range": 2}[kind]
        if _stream is not None:
            self.state = int(_stream(self.state, out, k, float(lo), float(hi)))
            return out
        from . import _native

        self.state = int(_native.lib().ct_rng_stream(self.state, 1, int(n), k, float(lo), float(hi),
                                                      out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

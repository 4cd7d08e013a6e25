"""Batched rendering of many scenes in one CUDA graph (ct_batch_*).

Each job is renderImage-equivalent: `spp` passes with frame indices
seed*7919 + k (tracer.ts:348-355), rendered together with every other job of
the batch. The per-job sums live in device tensors; `images()` returns the
means.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import _abi, _native
from .camera import CameraFrame
from .tracer import DeviceScene, TraceOptions


def divide_exact(sums, n: int):
    """sums / n in IEEE float32 division, as renderImage's final scale does.
    (torch turns division by a host scalar into a multiply by its rounded
    reciprocal, which can differ in the last bit.)"""
    import torch

    return sums / torch.full((), float(n), dtype=sums.dtype, device=sums.device)


@dataclass
class Job:
    scene: DeviceScene
    frame: CameraFrame
    width: int
    height: int
    spp: int
    seed: int = 0


class BatchRenderer:
    """All `jobs` rendered by one replayable graph. Scenes must outlive the renderer."""

    def __init__(self, jobs: Sequence[Job], opts: TraceOptions, wave_paths: int = 0, walk: int = -1):
        import torch

        self.jobs = list(jobs)
        self.opts = opts
        self._lib = _native.lib()
        self.accums = [torch.zeros(j.width * j.height * 3, dtype=torch.float32, device="cuda") for j in self.jobs]
        arr = (_abi.ct_batch_job * len(self.jobs))()
        for i, j in enumerate(self.jobs):
            arr[i].scene = j.scene.handle
            arr[i].frame = j.frame.struct()
            arr[i].width, arr[i].height = j.width, j.height
            arr[i].first_frame_index = (j.seed * 7919) & 0xFFFFFFFF
            arr[i].passes = j.spp
            arr[i].accum = self.accums[i].data_ptr()
        o = _abi.ct_trace_options(opts.max_bounces, int(opts.russian_roulette), int(opts.nee))
        handle = C.c_void_p()
        _native.check(self._lib.ct_batch_create(arr, len(self.jobs), C.byref(o), int(wave_paths), int(walk),
                                                C.byref(handle)))
        self.handle = handle

    def run(self, stream=None) -> None:
        """Adds every job's passes to its sums (graph launch; asynchronous)."""
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        _native.check(self._lib.ct_batch_run(self.handle, s))

    def set_first_frames(self, first: Sequence[int]) -> None:
        arr = (C.c_uint32 * len(self.jobs))(*[int(f) & 0xFFFFFFFF for f in first])
        _native.check(self._lib.ct_batch_set_first_frames(self.handle, arr))

    def reset(self) -> None:
        for a in self.accums:
            a.zero_()

    def images(self) -> List[np.ndarray]:
        """Mean radiance per job (sums / spp), float32 h*w*3, row 0 = top."""
        import torch

        torch.cuda.synchronize()
        return [divide_exact(a, j.spp).cpu().numpy() for a, j in zip(self.accums, self.jobs)]

    def info(self) -> dict:
        waves, nodes, walk = C.c_uint32(), C.c_uint64(), C.c_int32()
        paths = C.c_uint64()
        _native.check(self._lib.ct_batch_info(self.handle, C.byref(waves), C.byref(paths), C.byref(nodes),
                                              C.byref(walk)))
        return {"waves": waves.value, "paths": paths.value, "graph_nodes": nodes.value, "walk": walk.value}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._lib.ct_batch_destroy(self.handle)
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

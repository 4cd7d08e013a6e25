"""ct_accumulate_pass_noalloc: accumulatePass with its scratch in a static device array.

For callers that cannot allocate device memory while rendering (graph capture,
per-frame no-allocation rules, hosts that own all allocations). The entry
point must give the same samples as the allocating entry point, also on a
second call in a row, when the static array still holds the first call's data.
This file is collected last so a failure here stops a `-x` run only after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import caustic as ct
from caustic import _abi, _native

pytestmark = pytest.mark.gpu


def _pass_allocating(dev, frame, w, h, frame_index, opts):
    import torch

    acc = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    f = frame.struct()
    _native.check(dev._lib.ct_accumulate_passes_device(dev.handle, C.byref(f), w, h, frame_index, 1, C.byref(opts),
                                                       _native.ptr(acc), None, None))
    torch.cuda.synchronize()
    return acc.cpu().numpy()


def _pass_noalloc(dev, frame, w, h, frame_index, opts):
    import torch

    acc = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    f = frame.struct()
    _native.check(dev._lib.ct_accumulate_pass_noalloc(dev.handle, C.byref(f), w, h, frame_index, C.byref(opts),
                                                      _native.ptr(acc), None))
    torch.cuda.synchronize()
    return acc.cpu().numpy()


@pytest.mark.parametrize("scene_name", ["unit", "caustic"])
def test_noalloc_matches_allocating_entry_point_twice(native_lib, scene_name):
    if scene_name == "unit":
        sc, w, h = ct.cornell_unit_box(), 256, 256
    else:
        sc, w, h = ct.caustic_scene(level=4), 192, 108
    frame = ct.camera_frame(sc.camera, w / h)
    opts = _abi.ct_trace_options(8, 1, 1)
    with ct.DeviceScene.from_scene(sc) as dev:
        for frame_index in (7919, 7920):  # two calls in a row share the static scratch
            want = _pass_allocating(dev, frame, w, h, frame_index, opts)
            got = _pass_noalloc(dev, frame, w, h, frame_index, opts)
            assert np.isfinite(got).all() and got.sum() > 0
            assert np.allclose(got, want, rtol=1e-5, atol=1e-6)


def test_noalloc_rejects_images_beyond_its_scratch(native_lib):
    sc = ct.cornell_unit_box()
    frame = ct.camera_frame(sc.camera, 1.0)
    opts = _abi.ct_trace_options(8, 0, 1)
    with ct.DeviceScene.from_scene(sc) as dev:
        f = frame.struct()
        status = dev._lib.ct_accumulate_pass_noalloc(dev.handle, C.byref(f), 1024, 1024, 0, C.byref(opts),
                                                     C.c_void_p(16), None)
        assert status == 1
        assert b"exceeds the static scratch limit" in dev._lib.ct_last_error()

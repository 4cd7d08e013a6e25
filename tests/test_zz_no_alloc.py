"""ct_accumulate_pass_noalloc: accumulatePass with its scratch in a static device array.

For callers that cannot allocate device memory while rendering: real-time
loops with a no-allocation rule per frame, and plugin hosts that own every
allocation after load. The entry point must add exactly the samples the
allocating entry point adds (bit for bit: both run the same kernels on the
same pass), also on a second call in a row, when the static array still holds
the first call's data, and must add into the caller's sums rather than
overwrite them. This file is collected last so a failure here stops a `-x`
run only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import caustic as ct
from caustic import _abi, _native

pytestmark = pytest.mark.gpu

CT_OPT_PATH_KERNEL = 4  # include/caustic.h
LIMIT = 512  # CT_NOALLOC_MAX_PIXELS = 512 x 512


def _start(w, h):
    """Nonzero starting sums, the same for both entry points."""
    return np.random.default_rng(w * 7 + h).uniform(0.0, 2.0, w * h * 3).astype(np.float32)


def _pass_allocating(dev, frame, w, h, frame_index, opts, start):
    import torch

    acc = torch.from_numpy(start.copy()).cuda()
    f = frame.struct()
    _native.check(dev._lib.ct_accumulate_passes_device(dev.handle, C.byref(f), w, h, frame_index, 1, C.byref(opts),
                                                       _native.ptr(acc), None, None))
    torch.cuda.synchronize()
    return acc.cpu().numpy()


def _pass_noalloc(dev, frame, w, h, frame_index, opts, start):
    import torch

    acc = torch.from_numpy(start.copy()).cuda()
    f = frame.struct()
    _native.check(dev._lib.ct_accumulate_pass_noalloc(dev.handle, C.byref(f), w, h, frame_index, C.byref(opts),
                                                      _native.ptr(acc), None))
    torch.cuda.synchronize()
    return acc.cpu().numpy()


CASES = {
    # the headline Cornell configuration at the size limit: whole-path kernel, then the wavefront kernels
    "unit512_whole": ("unit", LIMIT, LIMIT, (8, 0, 1), 1),
    "unit512_wavefront": ("unit", LIMIT, LIMIT, (8, 0, 1), 0),
    "unit_roulette": ("unit", 256, 256, (8, 1, 1), 1),
    "unit_camera_rays_only": ("unit", 256, 200, (0, 0, 1), 0),
    "caustic": ("caustic", 192, 108, (12, 1, 1), 1),
}


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_equals_allocating_entry_point_twice(native_lib, case):
    scene_name, w, h, (bounces, rr, nee), path_kernel = CASES[case]
    sc = ct.cornell_unit_box() if scene_name == "unit" else ct.caustic_scene(level=4)
    frame = ct.camera_frame(sc.camera, w / h)
    opts = _abi.ct_trace_options(bounces, rr, nee)
    start = _start(w, h)
    with ct.DeviceScene.from_scene(sc) as dev:
        _native.check(dev._lib.ct_scene_set_option(dev.handle, CT_OPT_PATH_KERNEL, path_kernel))
        for frame_index in (7919, 7920):  # two calls in a row share the static scratch
            want = _pass_allocating(dev, frame, w, h, frame_index, opts, start)
            got = _pass_noalloc(dev, frame, w, h, frame_index, opts, start)
            assert np.isfinite(got).all() and (got - start).sum() > 0
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_images_beyond_its_scratch(native_lib):
    sc = ct.cornell_unit_box()
    frame = ct.camera_frame(sc.camera, 1.0)
    opts = _abi.ct_trace_options(8, 0, 1)
    with ct.DeviceScene.from_scene(sc) as dev:
        f = frame.struct()
        status = dev._lib.ct_accumulate_pass_noalloc(dev.handle, C.byref(f), LIMIT + 1, LIMIT, 0, C.byref(opts),
                                                     C.c_void_p(16), None)
        assert status == 1
        assert b"exceeds the static scratch limit" in dev._lib.ct_last_error()

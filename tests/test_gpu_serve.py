"""Serving with continuous batching on the device: every request's image is the
same alone and in the mix (bit for bit), equals its plain renderImage, and
admission under a tight device-memory budget changes nothing but timing."""
import numpy as np
import pytest

import caustic as ct
from caustic.serve import PATH_STATE_BYTES, STEPS_IN_FLIGHT, GpuExecutor, RenderServer, Request

pytestmark = pytest.mark.gpu

OPTS = ct.TraceOptions(max_bounces=6, russian_roulette=True, nee=True)


@pytest.fixture(scope="module")
def device_scenes(native_lib):
    scenes = {"cornell": ct.CORNELL_BOX, "unit": ct.cornell_unit_box(), "soup": ct.batch_scene(21, 5_000, 4),
              "caustic": ct.caustic_scene(level=3)}
    dev = {k: ct.DeviceScene.from_scene(v) for k, v in scenes.items()}
    yield scenes, dev
    for d in dev.values():
        d.close()


def _requests(scenes):
    shapes = [("cornell", 40, 30, 7), ("soup", 24, 24, 3), ("unit", 33, 17, 12), ("caustic", 48, 27, 5),
              ("cornell", 16, 16, 1), ("soup", 64, 48, 9), ("unit", 20, 20, 4), ("caustic", 31, 31, 2)]
    out = []
    for i, (name, w, h, spp) in enumerate(shapes):
        out.append(Request(i, name, ct.camera_frame(scenes[name].camera, w / h), w, h, spp, seed=3 + i))
    return out


def _serve(dev, reqs, **kw):
    srv = RenderServer(GpuExecutor(dev, OPTS), **kw)
    for r in reqs:
        srv.submit(r)
    srv.drain()
    return {r.request.rid: r.image for r in srv.results}, srv


def test_each_request_same_alone_and_in_the_mix(device_scenes):
    scenes, dev = device_scenes
    reqs = _requests(scenes)
    mixed, srv = _serve(dev, reqs, step_paths=6_000, max_passes_per_step=3)
    assert srv.steps > 4 and len(mixed) == len(reqs)
    for r in reqs:
        alone, _ = _serve(dev, [r], step_paths=50_000, max_passes_per_step=16)
        assert np.array_equal(alone[r.rid], mixed[r.rid]), r
        want = ct.render_image(dev[r.scene], r.frame, ct.RenderOptions(
            max_bounces=OPTS.max_bounces, russian_roulette=OPTS.russian_roulette, nee=OPTS.nee,
            width=r.width, height=r.height, spp=r.spp, seed=r.seed))
        assert np.isfinite(want).all()
        assert np.array_equal(mixed[r.rid].reshape(want.shape), want), r


def test_budget_limited_admission(device_scenes):
    scenes, dev = device_scenes
    reqs = _requests(scenes)
    free, _ = _serve(dev, reqs, step_paths=6_000, max_passes_per_step=3)
    step_paths = 6_000
    scene_bytes = sum(d.device_bytes for d in dev.values())
    budget = scene_bytes + STEPS_IN_FLIGHT * step_paths * PATH_STATE_BYTES + 2 * 64 * 48 * 12  # about two at a time
    tight, srv = _serve(dev, reqs, budget_bytes=budget, step_paths=step_paths, max_passes_per_step=3)
    assert srv.peak_bytes <= budget
    for r in reqs:
        assert np.array_equal(free[r.rid], tight[r.rid])


def test_run_direct_equals_graph_run(device_scenes):
    scenes, dev = device_scenes
    import ctypes as C

    import torch
    from caustic import _abi, _native

    lib = _native.lib()
    reqs = _requests(scenes)[:4]
    sums = []
    for direct in (False, True):
        bufs = [torch.zeros(r.pixels * 3, device="cuda") for r in reqs]
        arr = (_abi.ct_batch_job * len(reqs))()
        for k, r in enumerate(reqs):
            arr[k].scene = dev[r.scene].handle
            arr[k].frame = r.frame.struct()
            arr[k].width, arr[k].height = r.width, r.height
            arr[k].first_frame_index = r.seed * 7919
            arr[k].passes = r.spp
            arr[k].accum = bufs[k].data_ptr()
        h = C.c_void_p()
        _native.check(lib.ct_batch_create(arr, len(reqs), C.byref(OPTS.struct()), 2_000, -1, C.byref(h)))
        try:
            run = lib.ct_batch_run_direct if direct else lib.ct_batch_run
            _native.check(run(h, None))
            torch.cuda.synchronize()
        finally:
            lib.ct_batch_destroy(h)
        sums.append([b.cpu().numpy() for b in bufs])
    for a, b in zip(*sums):
        assert np.array_equal(a, b)


def test_per_frame_baseline_equals_plain(device_scenes):
    """The per-frame baseline (one accumulatePass per frame) and the plain
    renderImage baseline produce the same images: they differ in launch
    pattern only, which is what the served bench compares against."""
    from caustic.serve import render_per_frame, render_plain

    scenes, dev = device_scenes
    reqs = _requests(scenes)[:5]
    plain = {r.request.rid: r.image for r in render_plain(dev, reqs, OPTS)}
    frames = {r.request.rid: r.image for r in render_per_frame(dev, reqs, OPTS)}
    for r in reqs:
        assert np.array_equal(plain[r.rid], frames[r.rid]), r

"""GPU renders (ct_render_image / ct_accumulate_pass*) against the oracle.

Bars: furnace energy conservation to 1e-3 (naive paths are deterministic:
5 (1 - 0.8^65) per sample), the reference's furnace tolerances with NEE+MIS
and roulette, and per-pixel means within 3 combined standard errors of the
oracle's at equal spp (same seeds, same per-path random streams).
"""
import ctypes as C

import numpy as np
import pytest

import caustic as ct
from caustic import _abi, _native

pytestmark = pytest.mark.gpu


def gpu_sums(dev, frame, w, h, spp, seed, bounces, rr, nee):
    """Per-pixel sum and sum of squares over spp passes on the GPU."""
    import torch

    acc = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    sq = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    o = _abi.ct_trace_options(bounces, int(rr), int(nee))
    f = frame.struct()
    _native.check(dev._lib.ct_accumulate_passes_device(dev.handle, C.byref(f), w, h, seed * 7919, spp, C.byref(o),
                                                       _native.ptr(acc), _native.ptr(sq), None))
    torch.cuda.synchronize()
    return acc.cpu().numpy().astype(np.float64), sq.cpu().numpy().astype(np.float64)


def oracle_sums(oracle, packed, frame, w, h, spp, seed, bounces, rr, nee):
    opts = _abi.ct_render_options(w, h, spp, bounces, int(rr), int(nee), seed)
    mean, sumsq = oracle.render_image(packed, frame.struct(), opts, want_sumsq=True)
    return mean.astype(np.float64) * spp, sumsq


def three_sigma(gpu, ora, spp):
    (gs, gq), (os_, oq) = gpu, ora
    gm, om = gs / spp, os_ / spp
    gv = np.maximum(gq / spp - gm * gm, 0) / spp
    ov = np.maximum(oq / spp - om * om, 0) / spp
    se = np.sqrt(gv + ov)
    tol = 3 * se + 1e-4 * (1 + np.abs(om))
    bad = np.abs(gm - om) > tol
    return bad.mean(), gm, om


@pytest.fixture(scope="module")
def furnace(native_lib):
    sc = ct.furnace_scene()
    packed = ct.pack_scene(sc)
    with ct.DeviceScene(packed) as dev:
        yield packed, dev, ct.camera_frame(sc.camera, 1.0)


def test_furnace_energy_conservation(furnace):  # furnace.test.ts:28-43
    _, dev, frame = furnace
    img = ct.render_image(dev, frame, ct.RenderOptions(max_bounces=64, russian_roulette=False, nee=False,
                                                       width=8, height=8, spp=4096, seed=3))
    assert (np.abs(img - 5) / 5 < 0.05).all()
    exact = 5 * (1 - 0.8 ** 65)
    assert np.abs(img / exact - 1).max() < 1e-3


def test_furnace_nee_mis(furnace):  # furnace.test.ts:45-63
    _, dev, frame = furnace
    img = ct.render_image(dev, frame, ct.RenderOptions(max_bounces=64, russian_roulette=False, nee=True,
                                                       width=4, height=4, spp=4096, seed=9))
    assert abs(img.mean() - 5) / 5 < 0.03
    assert (np.abs(img - 5) / 5 < 0.08).all()


def test_furnace_roulette(furnace):  # furnace.test.ts:65-81
    _, dev, frame = furnace
    img = ct.render_image(dev, frame, ct.RenderOptions(max_bounces=64, russian_roulette=True, nee=False,
                                                       width=4, height=4, spp=4096, seed=5))
    assert abs(img.mean() - 5) / 5 < 0.03


def _lens_unit_box():
    """The benchmark box seen through a thin lens (radius 0.04, focused on the
    spheres): exercises the lens sample of the camera ray (camera.ts:62-72)."""
    import dataclasses

    sc = ct.cornell_unit_box()
    return dataclasses.replace(sc, camera=ct.camera_at((0, 0.5, 1.6), (0, 0.5, 0), 32, 0.04, 1.55))


def _with_sky(sc):
    """The scene under the reference's gradient sky (tracer.ts:39-47, 211-216)."""
    import dataclasses

    return dataclasses.replace(sc, sky=ct.SkyGradient((0.35, 0.55, 0.95), (1.0, 0.95, 0.85), 1.5))


SCENES = {"cornell": lambda: ct.CORNELL_BOX, "unit": ct.cornell_unit_box, "lens": _lens_unit_box,
          "caustic": lambda: ct.caustic_scene(level=4), "unit_sky": lambda: _with_sky(ct.cornell_unit_box()),
          "soup_sky": lambda: _with_sky(ct.batch_scene(5, 2_000, 4))}


@pytest.mark.parametrize("scene_name,w,h,spp,rr,bounces", [("cornell", 96, 64, 16, True, 8),
                                                            ("unit", 64, 64, 16, False, 8),
                                                            ("lens", 64, 64, 16, False, 8),
                                                            ("caustic", 96, 54, 16, True, 12),
                                                            ("unit_sky", 64, 64, 16, True, 8),
                                                            ("soup_sky", 64, 48, 16, True, 6)])
def test_three_sigma_agreement(oracle, native_lib, scene_name, w, h, spp, rr, bounces):
    sc = SCENES[scene_name]()
    packed = ct.pack_scene(sc)
    frame = ct.camera_frame(sc.camera, w / h)
    with ct.DeviceScene(packed) as dev:
        gpu = gpu_sums(dev, frame, w, h, spp, 1, bounces, rr, True)
    ora = oracle_sums(oracle, packed, frame, w, h, spp, 1, bounces, rr, True)
    frac_bad, gm, om = three_sigma(gpu, ora, spp)
    assert frac_bad <= 0.01, f"{frac_bad:.4f} of pixel channels outside 3 standard errors"
    assert abs(gm.mean() / om.mean() - 1) < 0.01


def test_cornell_reference_checks(native_lib):  # reference.test.ts:9-48 on the GPU render
    sc = ct.CORNELL_BOX
    with ct.DeviceScene.from_scene(sc) as dev:
        img = ct.render_image(dev, ct.camera_frame(sc.camera, 1.5),
                              ct.RenderOptions(width=96, height=64, spp=16, seed=1)).astype(np.float64)
    px = lambda x, y: img[(y * 96 + x) * 3:(y * 96 + x) * 3 + 3]
    assert np.isfinite(img).all() and img.sum() > 0
    lum = lambda p: 0.2126 * p[0] + 0.7152 * p[1] + 0.0722 * p[2]
    assert lum(px(48, 32)) > lum(px(0, 63))
    red = sum(px(x, y) for y in range(24, 40) for x in range(1, 7))
    green = sum(px(x, y) for y in range(24, 40) for x in range(89, 95))
    assert red[0] > 1.5 * red[1] and green[1] > 1.5 * green[0]


def test_accumulate_pass_is_a_sum(native_lib):  # tracer.ts:357-360
    sc = ct.cornell_unit_box()
    frame = ct.camera_frame(sc.camera, 1.0)
    with ct.DeviceScene.from_scene(sc) as dev:
        acc = np.zeros(32 * 32 * 3, np.float32)
        opts = ct.TraceOptions(max_bounces=8, russian_roulette=False, nee=True)
        for s in range(3):
            ct.accumulate_pass(dev, frame, 32, 32, 7919 * 4 + s, opts, acc)
        img = ct.render_image(dev, frame, ct.RenderOptions(max_bounces=8, russian_roulette=False, nee=True,
                                                           width=32, height=32, spp=3, seed=4))
    assert np.allclose(acc / 3, img, rtol=1e-5, atol=1e-6)


def test_render_sizes_and_waves(native_lib):
    """Odd sizes and a render split into several waves match single-pass sums."""
    sc = ct.cornell_unit_box()
    with ct.DeviceScene.from_scene(sc) as dev:
        for w, h in ((1, 1), (3, 5), (33, 17)):
            frame = ct.camera_frame(sc.camera, w / h)
            img = ct.render_image(dev, frame, ct.RenderOptions(width=w, height=h, spp=2, seed=2))
            assert img.shape == (w * h * 3,) and np.isfinite(img).all()


@pytest.mark.parametrize("scene_name", ["soup_sky", "caustic"])
def test_waves_on_several_streams_sum_in_pass_order(native_lib, scene_name):
    """A render split into many waves (consecutive waves on the caller's stream
    and the scene's side streams, their path state in separate sets) equals the
    same render in one wave bit for bit: every pixel's passes are still added
    in pass order. Sums of squares too."""
    import torch

    sc = SCENES[scene_name]()
    w, h, spp = 40, 24, 13
    frame = ct.camera_frame(sc.camera, w / h)
    o = _abi.ct_trace_options(8, 1, 1)
    f = frame.struct()
    with ct.DeviceScene.from_scene(sc) as dev:
        outs = []
        for wave_paths in (0, 2 * w * h, w * h):  # one wave; 7 waves of 2 passes; 13 waves of 1
            _native.check(dev._lib.ct_scene_set_option(dev.handle, 2, wave_paths))
            acc = torch.zeros(w * h * 3, device="cuda")
            sq = torch.zeros(w * h * 3, device="cuda")
            _native.check(dev._lib.ct_accumulate_passes_device(dev.handle, C.byref(f), w, h, 7919, spp, C.byref(o),
                                                               _native.ptr(acc), _native.ptr(sq), None))
            img = ct.render_image(dev, frame, ct.RenderOptions(width=w, height=h, spp=spp, seed=1))
            torch.cuda.synchronize()
            outs.append((acc.cpu().numpy(), sq.cpu().numpy(), img))
    for got in outs[1:]:
        for a, b in zip(outs[0], got):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))

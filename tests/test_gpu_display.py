"""Device tonemap / PPM (ct_tonemap_device, ct_ppm_device) and GPU picking
(ct_pick) against the oracle: bytes bit for bit, picks as the reference's walk."""
import pathlib

import numpy as np
import pytest

import caustic as ct
import oracle_lib as oracle
from test_gpu_trace import check_closest

pytestmark = pytest.mark.gpu
GOLDEN = pathlib.Path(__file__).parent / "golden"


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def test_device_ppm_reproduces_the_reference_golden(native_lib):
    """renderCornellReference's linear buffer (oracle) -> device PPM == out/cornell.ppm."""
    linear, _ = oracle.cornell_reference(96, 64, 16)
    ppm = ct.ppm_device(_dev(linear), 96, 64, 1, 0.0, "aces")
    assert ppm == (GOLDEN / "cornell.ppm").read_bytes()


@pytest.mark.parametrize("mode", ["aces", "reinhard"])
@pytest.mark.parametrize("samples,ev", [(1, 0.0), (3, 0.0), (16, 1.5), (7, -2.0), (0, 0.0)])
def test_tonemap_matches_oracle_on_wide_ranges(native_lib, mode, samples, ev):
    rng = np.random.default_rng(17 + samples)
    w, h = 37, 23
    acc = np.exp(rng.normal(-1.0, 3.0, w * h * 3)).astype(np.float32) * max(samples, 1)
    acc[::11] = 0.0
    acc[5::13] *= -1.0
    acc[7::101] = np.inf
    acc[9::103] = np.nan
    acc[3::97] = 3.0e38
    want = oracle.tonemap(acc, w, h, samples, ev, aces=mode == "aces")
    got = ct.tonemap_device(_dev(acc), w, h, samples, ev, mode).cpu().numpy()
    assert np.array_equal(got, want)


def _boundary_inputs(mode):
    """Float32 inputs around every rounding boundary k + 0.5 of 255 * srgb(map(x))."""
    from caustic.tonemap import aces_fitted, linear_to_srgb, reinhard

    f = aces_fitted if mode == "aces" else reinhard
    hi_x = 40.0 if mode == "aces" else 1e6
    lo = np.full(255, 1e-9)
    hi = np.full(255, hi_x)
    target = np.arange(255) + 0.5
    for _ in range(200):  # bisection on the monotone part of the curve
        mid = 0.5 * (lo + hi)
        above = linear_to_srgb(f(mid)) * 255 >= target
        hi = np.where(above, mid, hi)
        lo = np.where(above, lo, mid)
    x = hi.astype(np.float32)
    out = [x]
    for k in range(1, 4):
        out.append(np.nextafter(x, np.float32(np.inf)) if k == 1 else np.nextafter(out[-1], np.float32(np.inf)))
    down = x
    for _ in range(3):
        down = np.nextafter(down, np.float32(0))
        out.append(down)
    return np.concatenate(out)


@pytest.mark.parametrize("mode", ["aces", "reinhard"])
def test_tonemap_at_rounding_boundaries(native_lib, mode):
    x = _boundary_inputs(mode)
    acc = np.repeat(x, 3)
    n = len(x)
    want = oracle.tonemap(acc, n, 1, 1, 0.0, aces=mode == "aces")
    got = ct.tonemap_device(_dev(acc), n, 1, 1, 0.0, mode).cpu().numpy()
    assert np.array_equal(got, want)
    ppm = ct.ppm_device(_dev(acc), n, 1, 1, 0.0, mode)
    assert ppm == ct.encode_ppm(n, 1, want)


def test_tonemap_rejects_bad_arguments(native_lib):
    import ctypes as C

    from caustic import _native

    lib = _native.lib()
    a = _dev(np.zeros(12, np.float32))
    with pytest.raises(ct.CausticError):
        _native.check(lib.ct_tonemap_device(C.c_void_p(a.data_ptr()), 2, 2, 1.0, 0.0, 2, C.c_void_p(a.data_ptr()), None))
    size = C.c_uint64()
    with pytest.raises(ct.CausticError, match="PPM needs"):
        _native.check(lib.ct_ppm_device(C.c_void_p(a.data_ptr()), 2, 2, 1.0, 0.0, 0, C.c_void_p(a.data_ptr()), 10,
                                        C.byref(size), None))
    assert size.value == len(b"P6\n2 2\n255\n") + 12


def test_pick_glass_sphere_like_the_reference(native_lib):  # scenes.test.ts:94-104
    packed = ct.pack_scene(ct.CORNELL_BOX)
    frame = ct.camera_frame(ct.CORNELL_BOX.camera, 1.5)
    with ct.DeviceScene(packed) as dev:
        hit = ct.pick(dev, frame, 0.74, 0.15)
        assert hit is not None
        assert ct.CORNELL_BOX.objects[hit.object_index].name == "Glass sphere"
        assert hit.t > 1
    empty = ct.pack_scene(ct.Scene("empty", [], ct.CORNELL_BOX.camera))
    with ct.DeviceScene(empty) as dev:
        assert ct.pick(dev, frame, 0.5, 0.5) is None


def test_pick_grid_matches_the_oracle_walk(native_lib):
    scene = ct.caustic_scene(level=3)
    packed = ct.pack_scene(scene)
    frame = ct.camera_frame(scene.camera, 16 / 9)
    sx, sy = np.meshgrid(np.linspace(0, 1, 41), np.linspace(0, 1, 23))
    sx, sy = sx.ravel(), sy.ravel()
    rays = np.empty((len(sx), 8), np.float32)
    f = frame.struct()
    for i in range(len(sx)):
        r = np.zeros(6)
        oracle.lib().or_generate_ray(oracle.C.byref(f), sx[i], sy[i], 0.0, 0.0, oracle._p(r))
        rays[i, :6] = r
    rays[:, 6] = ct.T_MIN
    rays[:, 7] = np.inf
    with ct.DeviceScene(packed) as dev:
        obj, prim, t, point = ct.pick_many(dev, frame, sx, sy)
        check_closest(oracle, packed, rays, ct.Hits(prim, t), "pick")
    assert (prim >= 0).sum() > 0.5 * len(prim)
    hit = prim >= 0
    assert np.array_equal(obj[hit], packed.prim_object[prim[hit]])
    assert (obj[~hit] == -1).all() and np.isnan(point[~hit]).all()
    expect = rays[hit, :3].astype(np.float64) + rays[hit, 3:6].astype(np.float64) * t[hit, None]
    assert np.allclose(point[hit], expect, rtol=0, atol=1e-5)

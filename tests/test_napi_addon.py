"""The Node-API addon (caustic-tracer_gb300/napi/caustic_addon.c) on the CPU.

The addon is compiled against a recording stand-in for libcaustic_gb300 and
driven through a minimal Node-API implementation (tests/napi/), so these
tests check what the addon itself does: it maps the reference's objects
(PackedScene pack.ts:46-59, CameraFrame camera.ts:8-20, TraceOptions and
RenderOptions tracer.ts:27-31,337-342) onto the C structs, borrows typed
arrays without copying them, converts frameIndex and seed with ToUint32 as
rng.ts does, rejects wrong types (TypeError) and lengths (RangeError), and
turns a failed library call into an Error carrying the status name and the
library's message. The same addon against the real library is tested on the
GPU (test_gpu_napi_addon.py).
"""
import ctypes as C

import numpy as np
import pytest

import caustic as ct
from caustic import _abi
from napi_host import FAKE_ADDON, JsError, NodeHost, fake, frame_js, packed_scene_js


@pytest.fixture(scope="module")
def lib_fake():
    F = fake()
    F.fake_view.restype = C.POINTER(_abi.ct_packed_scene_view)
    F.fake_first_prim.restype = C.POINTER(C.c_float)
    F.fake_frame.restype = C.POINTER(_abi.ct_camera_frame)
    F.fake_render_options.restype = C.POINTER(_abi.ct_render_options)
    F.fake_trace_options.restype = C.POINTER(_abi.ct_trace_options)
    F.fake_fail_next.argtypes = [C.c_int, C.c_char_p]
    return F


@pytest.fixture(scope="module")
def cornell():
    sc = ct.CORNELL_BOX
    return ct.pack_scene(sc), ct.camera_frame(sc.camera, 1.5)


@pytest.fixture()
def node():
    with NodeHost(FAKE_ADDON) as host:
        yield host


def counts(F):
    a, b = C.c_int(), C.c_int()
    F.fake_counts(C.byref(a), C.byref(b))
    return a.value, b.value


def test_scene_create_borrows_the_packed_arrays(node, lib_fake, cornell):
    packed, _ = cornell
    js = packed_scene_js(packed)
    before = counts(lib_fake)
    scene = node.call("sceneCreate", js)
    v = lib_fake.fake_view().contents
    assert (v.prim_count, v.node_count, v.mat_count, v.light_count) == (
        packed.prim_count, packed.node_count, packed.mat_count, len(packed.lights))
    # zero copy: the library sees the typed arrays' own memory
    assert C.cast(v.prims, C.c_void_p).value == packed.prims.ctypes.data
    assert C.cast(v.nodes, C.c_void_p).value == packed.nodes.ctypes.data
    assert C.cast(v.lights, C.c_void_p).value == packed.lights.ctypes.data
    assert C.cast(v.prim_object, C.c_void_p).value == packed.prim_object.ctypes.data
    assert np.array_equal(np.ctypeslib.as_array(lib_fake.fake_first_prim(), (16,)), packed.prims[:16])
    assert v.sky.kind == 0
    assert counts(lib_fake)[0] == before[0] + 1
    # the handle's finalizer releases the scene once, at collection
    node.call("sceneDestroy", scene)
    node.call("sceneDestroy", scene)
    node.collect()
    assert counts(lib_fake)[1] == before[1] + 1


def test_gradient_sky_is_read(node, lib_fake, cornell):
    packed, _ = cornell
    js = packed_scene_js(packed)
    js["sky"] = {"kind": "gradient", "zenith": {"r": 0.1, "g": 0.2, "b": 0.3},
                 "horizon": {"r": 1.0, "g": 0.9, "b": 0.8}, "strength": 2.5}
    node.call("sceneCreate", js)
    sky = lib_fake.fake_view().contents.sky
    assert sky.kind == 1 and list(sky.zenith) == [0.1, 0.2, 0.3] and list(sky.horizon) == [1.0, 0.9, 0.8]
    assert sky.strength == 2.5


def test_render_image_maps_frame_and_options(node, lib_fake, cornell):
    packed, frame = cornell
    scene = node.call("sceneCreate", packed_scene_js(packed))
    opts = {"maxBounces": 6, "russianRoulette": False, "nee": True, "width": 12, "height": 5, "spp": 9, "seed": 3}
    img = node.call("renderImage", scene, frame_js(frame), opts).array()
    assert img.dtype == np.float32 and img.shape == (12 * 5 * 3,)
    assert np.array_equal(img, (np.arange(img.size) % 7).astype(np.float32) + np.float32(0.25 * 9))
    o = lib_fake.fake_render_options().contents
    assert (o.width, o.height, o.spp, o.max_bounces, o.russian_roulette, o.nee, o.seed) == (12, 5, 9, 6, 0, 1, 3)
    f = lib_fake.fake_frame().contents
    ref = frame.struct()
    for name in ("origin", "right", "up", "forward"):
        assert list(getattr(f, name)) == list(getattr(ref, name))
    assert (f.tan_half_fov, f.aspect, f.lens_radius, f.focus_distance) == (
        ref.tan_half_fov, ref.aspect, ref.lens_radius, ref.focus_distance)


@pytest.mark.parametrize("seed,want", [(None, 0), (0, 0), (1, 1), (-1, 4294967295), (2 ** 32 + 5, 5)])
def test_render_seed_is_to_uint32_with_default_0(node, lib_fake, cornell, seed, want):  # tracer.ts:351
    packed, frame = cornell
    scene = node.call("sceneCreate", packed_scene_js(packed))
    opts = {"maxBounces": 8, "russianRoulette": True, "nee": True, "width": 2, "height": 2, "spp": 1}
    if seed is not None:
        opts["seed"] = seed
    node.call("renderImage", scene, frame_js(frame), opts)
    assert lib_fake.fake_render_options().contents.seed == want


def test_accumulate_pass_adds_in_place(node, lib_fake, cornell):
    packed, frame = cornell
    scene = node.call("sceneCreate", packed_scene_js(packed))
    accum = np.full(4 * 3 * 3, 0.5, np.float32)
    topts = {"maxBounces": 3, "russianRoulette": True, "nee": False}
    node.call("accumulatePass", scene, frame_js(frame), 4, 3, 7919 * 2 + 3, topts, accum)
    assert np.all(accum == np.float32(0.5 + 1 + (7919 * 2 + 3) % 5))  # the caller's array, changed in place
    w, h, fi = C.c_int32(), C.c_int32(), C.c_uint32()
    lib_fake.fake_pass_args(C.byref(w), C.byref(h), C.byref(fi))
    assert (w.value, h.value, fi.value) == (4, 3, 7919 * 2 + 3)
    t = lib_fake.fake_trace_options().contents
    assert (t.max_bounces, t.russian_roulette, t.nee) == (3, 1, 0)
    node.call("accumulatePass", scene, frame_js(frame), 4, 3, -2.5, topts, accum)  # ToUint32(-2.5) = 2^32 - 2
    lib_fake.fake_pass_args(C.byref(w), C.byref(h), C.byref(fi))
    assert fi.value == 4294967294


def test_ray_queries(node, lib_fake, cornell):
    packed, _ = cornell
    scene = node.call("sceneCreate", packed_scene_js(packed))
    n = 37
    rays = np.zeros((n, 8), np.float32)
    rays[:, 7] = np.arange(n, dtype=np.float32) + 0.5
    prim, t = np.zeros(n, np.int32), np.zeros(n, np.float32)
    node.call("intersectClosestMany", scene, rays.reshape(-1), prim, t)
    assert np.array_equal(prim, np.arange(n) - 1) and np.array_equal(t, rays[:, 7])
    assert lib_fake.fake_rays() == n and lib_fake.fake_uv() == 0
    u, v = np.zeros(n, np.float32), np.zeros(n, np.float32)
    node.call("intersectClosestMany", scene, rays.reshape(-1), prim, t, u, v)
    assert lib_fake.fake_uv() == 1 and np.all(u == 0.25) and np.all(v == 0.5)
    blocked = np.zeros(n, np.uint8)
    node.call("occludedMany", scene, rays.reshape(-1), blocked)
    assert np.array_equal(blocked, np.arange(n) % 2)


def test_wrong_types_and_lengths_throw(node, cornell):
    packed, frame = cornell
    js = packed_scene_js(packed)
    bad = dict(js, prims=packed.prims.view(np.int32))
    with pytest.raises(JsError) as e:
        node.call("sceneCreate", bad)
    assert e.value.kind == "TypeError" and "prims" in e.value.message
    with pytest.raises(JsError) as e:
        node.call("sceneCreate", dict(js, primCount=packed.prim_count + 1))
    assert e.value.kind == "RangeError"
    with pytest.raises(JsError) as e:
        node.call("sceneCreate", dict(js, sky={"kind": "starfield"}))
    assert e.value.kind == "RangeError"
    scene = node.call("sceneCreate", js)
    f = frame_js(frame)
    with pytest.raises(JsError) as e:  # maxBounces missing: undefined is not a number
        node.call("renderImage", scene, f, {"russianRoulette": True, "nee": True, "width": 2, "height": 2, "spp": 1})
    assert e.value.kind == "TypeError" and "maxBounces" in e.value.message
    with pytest.raises(JsError) as e:
        node.call("renderImage", scene, f, {"maxBounces": 8, "russianRoulette": 1, "nee": True, "width": 2,
                                            "height": 2, "spp": 1})
    assert e.value.kind == "TypeError" and "russianRoulette" in e.value.message
    with pytest.raises(JsError) as e:
        node.call("renderImage", scene, f, {"maxBounces": 8, "russianRoulette": True, "nee": True, "width": 2.5,
                                            "height": 2, "spp": 1})
    assert e.value.kind == "RangeError"
    topts = {"maxBounces": 8, "russianRoulette": True, "nee": True}
    with pytest.raises(JsError) as e:
        node.call("accumulatePass", scene, f, 4, 4, 0, topts, np.zeros(4 * 4 * 3 - 1, np.float32))
    assert e.value.kind == "RangeError" and "accum" in e.value.message
    with pytest.raises(JsError) as e:
        node.call("accumulatePass", scene, f, 4, 4, 0, topts, np.zeros(4 * 4 * 3, np.float64))
    assert e.value.kind == "TypeError"
    with pytest.raises(JsError) as e:
        node.call("intersectClosestMany", scene, np.zeros(12, np.float32), np.zeros(1, np.int32),
                  np.zeros(1, np.float32))
    assert e.value.kind == "RangeError"
    with pytest.raises(JsError) as e:
        node.call("renderImage", {"not": "a scene"}, f, {})
    assert e.value.kind == "TypeError" and "scene" in e.value.message
    with pytest.raises(JsError) as e:
        node.call("accumulatePass", scene, f)
    assert e.value.kind == "TypeError"


def test_library_failures_become_errors_with_the_status_name(node, lib_fake, cornell):
    packed, frame = cornell
    lib_fake.fake_fail_next(1, b"node 3: skip link 99 beyond node count 7")
    with pytest.raises(JsError) as e:
        node.call("sceneCreate", packed_scene_js(packed))
    assert (e.value.kind, e.value.code) == ("Error", "CT_ERR_INVALID_ARGUMENT")
    assert e.value.message == "node 3: skip link 99 beyond node count 7"
    scene = node.call("sceneCreate", packed_scene_js(packed))
    lib_fake.fake_fail_next(2, b"cudaErrorLaunchFailure")
    with pytest.raises(JsError) as e:
        node.call("renderImage", scene, frame_js(frame),
                  {"maxBounces": 8, "russianRoulette": True, "nee": True, "width": 2, "height": 2, "spp": 1})
    assert e.value.code == "CT_ERR_CUDA" and "cudaErrorLaunchFailure" in e.value.message
    node.call("sceneDestroy", scene)
    with pytest.raises(JsError) as e:
        node.call("renderImage", scene, frame_js(frame),
                  {"maxBounces": 8, "russianRoulette": True, "nee": True, "width": 2, "height": 2, "spp": 1})
    assert e.value.kind == "RangeError" and "destroyed" in e.value.message


def test_real_addon_exports_the_module_entry_points(native_lib):
    """The product addon (built with the library) loads through Node's entry point and exports the surface."""
    import subprocess

    from napi_host import REAL_ADDON

    assert REAL_ADDON.exists()
    out = subprocess.run(["nm", "-D", "--defined-only", str(REAL_ADDON)], capture_output=True, text=True).stdout
    assert "napi_register_module_v1" in out and "node_api_module_get_api_version_v1" in out
    with NodeHost(REAL_ADDON) as host:
        assert host.S.stub_kind(host.exports) == 5  # the exports object
        for name in ("sceneCreate", "sceneDestroy", "renderImage", "accumulatePass", "intersectClosestMany",
                     "occludedMany"):
            with pytest.raises(JsError) as e:  # called without arguments: a TypeError, not a crash
                host.call(name)
            assert e.value.kind == "TypeError"

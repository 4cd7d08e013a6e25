"""The Node-API addon against the real library on the GPU.

The product addon (caustic-tracer_gb300/_build/caustic_addon.node, linked to
libcaustic_gb300.so) is loaded through the minimal Node-API host of the tests
as Node would load it, and driven with the reference's objects: renderImage
(tracer.ts:348-355), accumulatePass (tracer.ts:361-395) and the batched
intersectClosest / occluded (intersect.ts:202-282, 368-420) give the same
bits as the same calls made directly through the C ABI, and a malformed
PackedScene is rejected with the library's status and message.
"""
import numpy as np
import pytest

import caustic as ct
from napi_host import REAL_ADDON, JsError, NodeHost, frame_js, packed_scene_js

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def host(native_lib):
    with NodeHost(REAL_ADDON) as h:
        yield h


def test_render_image_and_accumulate_pass_through_the_addon(host):
    sc = ct.CORNELL_BOX
    w, h = 64, 48
    packed = ct.pack_scene(sc)
    frame = ct.camera_frame(sc.camera, w / h)
    scene = host.call("sceneCreate", packed_scene_js(packed))
    opts = {"maxBounces": 8, "russianRoulette": True, "nee": True, "width": w, "height": h, "spp": 8, "seed": 1}
    img = host.call("renderImage", scene, frame_js(frame), opts).array()
    with ct.DeviceScene(packed) as dev:
        want = ct.render_image(dev, frame, ct.RenderOptions(max_bounces=8, russian_roulette=True, nee=True, width=w,
                                                            height=h, spp=8, seed=1))
        acc_direct = np.full(w * h * 3, 0.25, np.float32)
        ct.accumulate_pass(dev, frame, w, h, 7919 + 3, ct.TraceOptions(8, False, True), acc_direct)
    assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
    acc = np.full(w * h * 3, 0.25, np.float32)
    host.call("accumulatePass", scene, frame_js(frame), w, h, 7919 + 3,
              {"maxBounces": 8, "russianRoulette": False, "nee": True}, acc)
    assert np.array_equal(acc.view(np.uint32), acc_direct.view(np.uint32))
    host.call("sceneDestroy", scene)


def test_ray_queries_through_the_addon(host, oracle):
    packed = ct.pack_scene(ct.random_test_scene(ct.Rng(1234), 300, 600))
    rays = ct.soup_rays(50_000, seed=3, radius=14.0, half=8.0)
    scene = host.call("sceneCreate", packed_scene_js(packed))
    n = len(rays)
    prim, t = np.zeros(n, np.int32), np.zeros(n, np.float32)
    u, v = np.zeros(n, np.float32), np.zeros(n, np.float32)
    host.call("intersectClosestMany", scene, rays.reshape(-1), prim, t, u, v)
    blocked = np.zeros(n, np.uint8)
    shadow = rays.copy()
    shadow[:, 7] = 5.0
    host.call("occludedMany", scene, shadow.reshape(-1), blocked)
    with ct.DeviceScene(packed) as dev:
        want = ct.intersect_closest(dev, rays, barycentrics=True)
        want_blocked = ct.occluded(dev, shadow)
    assert np.array_equal(prim, want.prim) and np.array_equal(t.view(np.uint32), want.t.view(np.uint32))
    assert np.array_equal(u.view(np.uint32), want.u.view(np.uint32))
    assert np.array_equal(blocked.astype(bool), want_blocked)
    assert np.array_equal(blocked.astype(bool), oracle.occluded(packed, shadow)[0])
    host.call("sceneDestroy", scene)


def test_malformed_scene_is_rejected_with_the_library_status(host):
    packed = ct.pack_scene(ct.random_test_scene(ct.Rng(7), 20, 20))
    js = packed_scene_js(packed)
    nodes = packed.nodes.copy()
    nodes[3] = 1e6  # skip link of the root far beyond the node count
    js["nodes"] = nodes
    with pytest.raises(JsError) as e:
        host.call("sceneCreate", js)
    assert (e.value.kind, e.value.code) == ("Error", "CT_ERR_INVALID_ARGUMENT")
    assert e.value.message


def test_scene_handles_are_released_by_their_finalizer(host):
    packed = ct.pack_scene(ct.cornell_unit_box())
    for _ in range(3):
        host.call("sceneCreate", packed_scene_js(packed))
    assert host.collect() >= 3

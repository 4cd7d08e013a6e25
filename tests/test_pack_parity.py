"""The library's host packer (ct_pack_scene) against the oracle's packScene.

Both restate pack.ts/bvh.ts independently; their arrays must be identical
bit for bit on every scene shape the reference supports.
"""
import numpy as np
import pytest

import caustic as ct
from caustic.scene import Lambertian, Mesh, Scene, SceneObject, Sphere, Triangle


def _same(a, b):
    assert a.prim_count == b.prim_count and a.node_count == b.node_count and a.mat_count == b.mat_count
    for name in ("prims", "nodes", "mats", "lights", "prim_object", "order"):
        x, y = getattr(a, name), getattr(b, name)
        assert x.dtype == y.dtype and x.shape == y.shape, name
        assert np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y), name


def test_cornell_preset_matches_oracle(oracle):
    want, cam = oracle.pack_cornell()
    got = ct.pack_scene(ct.CORNELL_BOX)
    _same(got, want)
    assert got.prim_count == 12 + 2
    # scenes.test.ts:44-52: the ceiling light is the only emitter
    objs = {int(got.prim_object[p]) for p in got.lights}
    assert [ct.CORNELL_BOX.objects[o].name for o in objs] == ["Ceiling light"]
    c = ct.CORNELL_BOX.camera
    assert (c.yaw, c.pitch, c.distance, c.fov_deg) == (cam.yaw, cam.pitch, cam.distance, cam.fov_deg)


@pytest.mark.parametrize("name", ["random", "furnace", "unit_cornell", "soup", "caustic_small", "empty",
                                  "coincident", "mixed_mesh"])
def test_scene_matches_oracle(oracle, name):
    if name == "random":
        scene = ct.random_test_scene(ct.Rng(1234), 1000, 2000)
    elif name == "furnace":
        scene = ct.furnace_scene()
    elif name == "unit_cornell":
        scene = ct.cornell_unit_box()
    elif name == "soup":
        scene = ct.triangle_soup(20_000, seed=11)
    elif name == "caustic_small":
        scene = ct.caustic_scene(level=4)
    elif name == "empty":
        scene = Scene("empty", [], ct.CORNELL_BOX.camera)
    elif name == "coincident":
        scene = Scene("c", [SceneObject(f"c{i}", "c", Sphere((1, 2, 3), 0.5), Lambertian((1, 1, 1)))
                            for i in range(40)], ct.CORNELL_BOX.camera)
    else:
        verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float64)
        idx = np.array([0, 1, 2, 0, 2, 3, 1, 2, 4, 2, 3, 4], np.uint32)
        objs = [SceneObject("m", "m", Mesh(verts, idx), ct.Metal((0.9, 0.8, 0.7), 0.1)),
                SceneObject("t", "t", Triangle((2, 0, 0), (3, 0, 0), (2, 1, 0)), ct.Emissive((1, 1, 1), 4)),
                SceneObject("s", "s", Sphere((0, 3, 0), 0.5), ct.Dielectric(1.33, (0.9, 1, 0.9))),
                SceneObject("q", "q", ct.Quad((-1, -1, -1), (2, 0, 0), (0, 0, 2)),
                            Lambertian((0.5, 0.5, 0.5), ct.CheckerTexture((0.1, 0.1, 0.1), 3.0), (0.2, 0, 0)))]
        scene = Scene("mixed", objs, ct.CORNELL_BOX.camera, ct.SkyGradient((0.5, 0.7, 1), (1, 1, 1), 1))
    got = ct.pack_scene(scene)
    want = oracle.pack(scene)
    _same(got, want)
    rep = oracle.validate(got)
    assert rep["ok"], rep


def test_packed_arrays_finite_and_sized():
    # scenes.test.ts:18-33
    ps = ct.pack_scene(ct.caustic_scene(level=3))
    for arr in (ps.prims, ps.nodes, ps.mats):
        assert np.isfinite(arr).all()
    assert len(ps.mats) == ps.mat_count * 16


def test_pack_rejects_bad_input():
    bad = Scene("bad", [SceneObject("m", "m", Mesh(np.zeros((2, 3)), np.array([0, 1, 5], np.uint32)),
                                    Lambertian((1, 1, 1)))], ct.CORNELL_BOX.camera)
    with pytest.raises(ct.CausticError, match="out of range"):
        ct.pack_scene(bad)

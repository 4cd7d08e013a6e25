"""bvh.test.ts restated against the oracle (and the host packer's arrays).

Random scene of 1000 spheres + 2000 triangles from Rng(1234); rays from
Rng(99) / Rng(5) / Rng(7) exactly as the reference test draws them.
"""
import math

import numpy as np
import pytest

from caustic import Rng, pack_scene, random_test_scene
from caustic.scene import Lambertian, Scene, SceneObject, Sphere


@pytest.fixture(scope="module")
def packed():
    return pack_scene(random_test_scene(Rng(1234), 1000, 2000))


def closest_rays_99(n=1000):  # bvh.test.ts:89-99
    r = Rng(99)
    rays = np.zeros((n, 8), np.float32)
    for i in range(n):
        o = (r.range(-14, 14), r.range(-14, 14), r.range(-14, 14))
        t = (r.range(-8, 8), r.range(-8, 8), r.range(-8, 8))
        d = (t[0] - o[0], t[1] - o[1], t[2] - o[2])
        length = math.hypot(*d)
        rays[i] = (*o, *(c / length for c in d), 1e-4, np.inf)
    return rays


def finite_tmax_rays(seed, n, lo_t, hi_t, span=12):  # bvh.test.ts:114-146
    r = Rng(seed)
    rays = np.zeros((n, 8), np.float32)
    for i in range(n):
        o = (r.range(-span, span), r.range(-span, span), r.range(-span, span))
        d = (r.range(-1, 1), r.range(-1, 1), r.range(-1, 1))
        length = math.hypot(*d) or 1
        tmax = r.range(lo_t, hi_t)
        rays[i] = (*o, *(c / length for c in d), 1e-4, tmax)
    return rays


def test_packs_every_primitive(packed):  # bvh.test.ts:50-54
    assert packed.prim_count == 3000
    assert packed.node_count > 1
    assert len(packed.nodes) == packed.node_count * 8


def test_leaves_at_most_four(packed):  # bvh.test.ts:56-67
    leaf = packed.nodes[7::8]
    words = leaf[leaf >= 0].astype(np.int64)
    assert ((words & 7) <= 4).all() and ((words & 7) > 0).all()
    assert len(words) >= math.ceil(3000 / 4)


def test_skip_links_valid(oracle, packed):  # bvh.test.ts:69-80
    rep = oracle.validate(packed)
    assert rep["ok"] and rep["errors"] == 0 and rep["max_leaf"] <= 4
    skip = packed.nodes[3::8]
    idx = np.arange(packed.node_count)
    assert (skip > idx).all() and (skip <= packed.node_count).all()


@pytest.mark.parametrize("mode", [0, 1], ids=["ordered", "stackless"])
def test_traversal_matches_brute_force(oracle, packed, mode):  # bvh.test.ts:88-112
    rays = closest_rays_99()
    p, t, u, v, _ = oracle.trace(packed, rays, mode)
    bp, bt, bu, bv, _ = oracle.trace(packed, rays, 2)
    assert np.array_equal(p, bp)
    hit = p >= 0
    assert hit.sum() > 500
    assert np.abs(t[hit] - bt[hit]).max() < 1e-6
    tri = hit & (packed.prims[p.clip(0) * 16 + 3] == 1)
    assert np.abs(u[tri] - bu[tri]).max() < 1e-9 and np.abs(v[tri] - bv[tri]).max() < 1e-9


@pytest.mark.parametrize("mode", [0, 1], ids=["ordered", "stackless"])
def test_finite_tmax(oracle, packed, mode):  # bvh.test.ts:114-131
    rays = finite_tmax_rays(5, 300, 0.5, 20)
    p, t, *_ = oracle.trace(packed, rays, mode)
    bp, *_ = oracle.trace(packed, rays, 2)
    assert np.array_equal(p, bp)
    assert (t[p >= 0] < rays[p >= 0, 7]).all()


def test_occlusion_matches_brute_force(oracle, packed):  # bvh.test.ts:134-146
    rays = finite_tmax_rays(7, 500, 1, 30)
    blocked, _ = oracle.occluded(packed, rays)
    bp, *_ = oracle.trace(packed, rays, 2)
    assert np.array_equal(blocked, bp >= 0)


def test_degenerate_inputs(oracle, packed):  # bvh.test.ts:148-169
    base = random_test_scene(Rng(1234), 0, 0)
    empty = pack_scene(Scene("empty", [], base.camera))
    assert empty.prim_count == 0
    ray = np.array([[0, 0, 0, 0, 0, 1, 1e-4, np.inf]], np.float32)
    p, *_ = oracle.trace(empty, ray, 0)
    assert p[0] == -1
    same = [SceneObject(f"c{i}", "c", Sphere((1, 2, 3), 0.5), Lambertian((1, 1, 1))) for i in range(40)]
    co = pack_scene(Scene("coincident", same, base.camera))
    rep = oracle.validate(co)
    assert rep["ok"] and rep["max_leaf"] <= 4
    p, t, *_ = oracle.trace(co, np.array([[1, 2, -5, 0, 0, 1, 1e-4, np.inf]], np.float32), 0)
    assert p[0] >= 0 and abs(t[0] - 7.5) < 1e-5


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_leaves_in_node_order_cover_primitives_in_packed_order(seed):
    """The stackless walk visits leaves in node-array order; they must cover
    the primitives contiguously in packed order (the GPU's small-scene form
    tests primitives in that order and relies on it)."""
    import caustic as ct

    scenes = [ct.CORNELL_BOX, ct.cornell_unit_box(), ct.random_test_scene(ct.Rng(seed), 10 * seed, 20 * seed),
              ct.batch_scene(seed, 40 * seed, 3 * seed)]
    for sc in scenes:
        p = ct.pack_scene(sc)
        nodes = np.asarray(p.nodes).reshape(-1, 8)
        nxt = 0
        for row in nodes:
            if row[7] >= 0:
                word = int(row[7])
                assert word >> 3 == nxt, sc.name
                nxt += word & 7
        assert nxt == p.prim_count, sc.name

"""GPU ray queries (ct_trace_closest / ct_trace_occluded) against the oracle.

Parity bar: the hit primitive index equals the reference's (the oracle's
float64 ordered walk) bit for bit, except at ties, where the GPU's primitive
must itself be hit (in float64) at a distance within 1e-5 relative of the
reference's closest t. Misses and occlusion flags must match exactly.
"""
import numpy as np
import pytest

import caustic as ct
from test_oracle_bvh import closest_rays_99, finite_tmax_rays

pytestmark = pytest.mark.gpu
TIE_REL = 1e-5


def check_closest(oracle, packed, rays, hits, label=""):
    p, t, u, v, _ = oracle.trace(packed, rays, 0)
    assert np.array_equal(p < 0, hits.prim < 0), f"{label}: hit/miss differs"
    diff = np.nonzero(p != hits.prim)[0]
    for i in diff:
        t_gpu_prim = oracle.prim_hit_t(packed, int(hits.prim[i]), rays[i])
        assert t_gpu_prim > 0, f"{label}: ray {i}: GPU prim {hits.prim[i]} is not hit in float64"
        assert abs(t_gpu_prim - t[i]) <= TIE_REL * t[i], f"{label}: ray {i}: not a tie ({t_gpu_prim} vs {t[i]})"
    hit = p >= 0
    if hit.any():
        rel = np.abs(hits.t[hit].astype(np.float64) - t[hit]) / t[hit]
        assert rel.max() <= 4e-6, f"{label}: t relative error {rel.max()}"  # the reported bound, kTRel
    assert np.isinf(hits.t[~hit]).all()
    return len(diff), int(hit.sum())


@pytest.fixture(scope="module")
def random_scene(native_lib):
    packed = ct.pack_scene(ct.random_test_scene(ct.Rng(1234), 1000, 2000))
    with ct.DeviceScene(packed) as dev:
        yield packed, dev


@pytest.mark.parametrize("variant", ["ordered", "stackless", "ordered_thread"])
def test_closest_matches_reference_rays(oracle, random_scene, variant):  # bvh.test.ts:88-112
    packed, dev = random_scene
    prev = ct.set_traversal(variant)
    try:
        rays = closest_rays_99()
        hits = ct.intersect_closest(dev, rays, barycentrics=True)
        ties, n_hit = check_closest(oracle, packed, rays, hits, variant)
        assert n_hit > 500 and ties == 0
        p, t, u, v, _ = oracle.trace(packed, rays, 0)
        tri = (p >= 0) & (packed.prims[p.clip(0) * 16 + 3] == 1)
        assert np.abs(hits.u[tri] - u[tri]).max() < 1e-5
        assert np.abs(hits.v[tri] - v[tri]).max() < 1e-5
    finally:
        ct.set_traversal(prev)


@pytest.mark.parametrize("variant", ["ordered", "stackless", "ordered_thread"])
def test_closest_many_rays_and_finite_tmax(oracle, random_scene, variant):  # bvh.test.ts:114-131
    packed, dev = random_scene
    prev = ct.set_traversal(variant)
    try:
        r = ct.Rng(2024)
        n = 200_000
        u = r.draw(n * 6).reshape(n, 6)
        o = -14 + 28 * u[:, :3]
        d = (-8 + 16 * u[:, 3:]) - o
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays = ct.make_rays(o, d)
        hits = ct.intersect_closest(dev, rays)
        check_closest(oracle, packed, rays, hits, "200k")
        rays = finite_tmax_rays(5, 300, 0.5, 20)
        hits = ct.intersect_closest(dev, rays)
        check_closest(oracle, packed, rays, hits, "tmax")
        assert (hits.t[hits.prim >= 0] < rays[hits.prim >= 0, 7]).all()
    finally:
        ct.set_traversal(prev)


@pytest.mark.parametrize("variant", ["ordered", "stackless", "ordered_thread"])
def test_occluded_matches_reference(oracle, random_scene, variant):  # bvh.test.ts:134-146
    packed, dev = random_scene
    prev = ct.set_traversal(variant)
    try:
        rays = finite_tmax_rays(7, 500, 1, 30)
        assert np.array_equal(ct.occluded(dev, rays), oracle.occluded(packed, rays)[0])
        rays = finite_tmax_rays(8, 100_000, 0.01, 30, span=14)
        assert np.array_equal(ct.occluded(dev, rays), oracle.occluded(packed, rays)[0])
    finally:
        ct.set_traversal(prev)


def test_triangle_soup_parity(oracle, native_lib):
    packed = ct.pack_scene(ct.triangle_soup(100_000, seed=5))
    rays = ct.soup_rays(500_000, seed=6)
    with ct.DeviceScene(packed) as dev:
        hits = ct.intersect_closest(dev, rays)
        ties, n_hit = check_closest(oracle, packed, rays, hits, "soup")
        assert n_hit > 0.5 * len(rays)
        assert ties <= 50


def test_degenerate_scenes(oracle, native_lib):  # bvh.test.ts:148-169
    from caustic.scene import Lambertian, Scene, SceneObject, Sphere

    cam = ct.CORNELL_BOX.camera
    empty = ct.pack_scene(Scene("empty", [], cam))
    with ct.DeviceScene(empty) as dev:
        hits = ct.intersect_closest(dev, np.array([[0, 0, 0, 0, 0, 1, 1e-4, np.inf]], np.float32))
        assert hits.prim[0] == -1 and np.isinf(hits.t[0])
    same = [SceneObject(f"c{i}", "c", Sphere((1, 2, 3), 0.5), Lambertian((1, 1, 1))) for i in range(40)]
    co = ct.pack_scene(Scene("c", same, cam))
    with ct.DeviceScene(co) as dev:
        hits = ct.intersect_closest(dev, np.array([[1, 2, -5, 0, 0, 1, 1e-4, np.inf]], np.float32))
        assert hits.prim[0] >= 0 and abs(hits.t[0] - 7.5) < 1e-5
    one = ct.pack_scene(Scene("one", same[:1], cam))  # the root is a leaf
    with ct.DeviceScene(one) as dev:
        hits = ct.intersect_closest(dev, np.array([[1, 2, -5, 0, 0, 1, 1e-4, np.inf],
                                                   [1, 2, 3, 0, 0, 1, 1e-4, np.inf],
                                                   [9, 9, 9, 0, 0, 1, 1e-4, np.inf]], np.float32))
        assert list(hits.prim) == [0, 0, -1]
        assert abs(hits.t[0] - 7.5) < 1e-5 and abs(hits.t[1] - 0.5) < 1e-6


def test_ragged_batch_sizes(oracle, random_scene):
    packed, dev = random_scene
    rays_all = closest_rays_99(1000)
    for n in (0, 1, 31, 32, 33, 127, 128, 129, 999):
        hits = ct.intersect_closest(dev, rays_all[:n])
        assert len(hits.prim) == n
        if n:
            check_closest(oracle, packed, rays_all[:n], hits, f"n={n}")



def _grazing_case(offset, n=60_000, seed=31):
    """Large, thin and small triangles around `offset`, hit by rays that graze
    them (direction nearly in the triangles' plane) and by ordinary rays."""
    from caustic.scene import Lambertian, Mesh, Scene, SceneObject

    rng = np.random.default_rng(seed)
    tris = []
    for k in range(400):
        size = 10.0 ** rng.uniform(-3, 1)
        centre = offset + rng.uniform(-5, 5, 3)
        e1 = rng.normal(size=3)
        e2 = rng.normal(size=3) * (10.0 ** rng.uniform(-3, 0))  # some thin triangles
        tris.append([centre, centre + size * e1, centre + size * e2])
    verts = np.asarray(tris, np.float64).reshape(-1, 3)
    mesh = Mesh(verts, np.arange(len(verts), dtype=np.uint32))
    scene = Scene("grazing", [SceneObject("m", "m", mesh, Lambertian((0.5, 0.5, 0.5)))], ct.CORNELL_BOX.camera)
    packed = ct.pack_scene(scene)
    pick = rng.integers(0, len(tris), n)
    t = np.asarray(tris)[pick]
    bary = rng.dirichlet((1, 1, 1), n)
    target = (bary[:, :, None] * t).sum(1)
    normal = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    normal /= np.linalg.norm(normal, axis=1, keepdims=True)
    inplane = np.cross(normal, rng.normal(size=(n, 3)))
    inplane /= np.linalg.norm(inplane, axis=1, keepdims=True)
    tilt = 10.0 ** rng.uniform(-5, 0, n)[:, None]  # cos(angle to the plane) from 1e-5 to 1
    d = inplane * np.sqrt(1 - tilt ** 2) + normal * tilt
    dist = 10.0 ** rng.uniform(-1, 2, n)[:, None]
    origin = target - d * dist
    return packed, ct.make_rays(origin.astype(np.float32), d.astype(np.float32))


@pytest.mark.parametrize("offset", [0.0, 3000.0])
def test_reported_distance_bound_holds_on_grazing_and_far_geometry(oracle, native_lib, offset):
    packed, rays = _grazing_case(np.array([offset, -offset / 3, offset / 7]))
    with ct.DeviceScene(packed) as dev:
        hits = ct.intersect_closest(dev, rays)
        ties, n_hit = check_closest(oracle, packed, rays, hits, f"grazing@{offset}")
        assert n_hit > 0.5 * len(rays)
        with_bary = ct.intersect_closest(dev, rays, barycentrics=True)  # the float64 refine path
        check_closest(oracle, packed, rays, with_bary, f"grazing@{offset}+uv")


def test_pipelined_host_queries_equal_device_queries(native_lib):
    """Host-pointer batches of more than two chunks (4 Mi rays each) are
    copied in, traced and copied out in overlapping chunks; the answers equal
    the device-pointer call's on the same rays, the ragged last chunk too."""
    import ctypes as C

    import torch
    from caustic import _native

    packed = ct.pack_scene(ct.triangle_soup(20_000, seed=9))
    n = 2 * (1 << 22) + 12_345
    rays = ct.soup_rays(n, seed=21)
    with ct.DeviceScene(packed) as dev:
        host = ct.intersect_closest(dev, rays, barycentrics=True)
        assert host.stats.launches == 3
        blocked = ct.occluded(dev, rays)
        lib = _native.lib()
        d_rays = torch.from_numpy(rays).cuda()
        d_p = torch.empty(n, dtype=torch.int32, device="cuda")
        d_t, d_u, d_v = (torch.empty(n, device="cuda") for _ in range(3))
        _native.check(lib.ct_trace_closest_device(dev.handle, _native.ptr(d_rays), n, _native.ptr(d_p),
                                                  _native.ptr(d_t), _native.ptr(d_u), _native.ptr(d_v), None))
        d_b = torch.empty(n, dtype=torch.uint8, device="cuda")
        _native.check(lib.ct_trace_occluded_device(dev.handle, _native.ptr(d_rays), n, _native.ptr(d_b), None))
        torch.cuda.synchronize()
        assert np.array_equal(host.prim, d_p.cpu().numpy())
        for a, b in ((host.t, d_t), (host.u, d_u), (host.v, d_v)):
            assert np.array_equal(a.view(np.uint32), b.cpu().numpy().view(np.uint32))
        assert np.array_equal(blocked.astype(np.uint8), d_b.cpu().numpy())

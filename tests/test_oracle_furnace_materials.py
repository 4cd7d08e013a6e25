"""furnace.test.ts and materials.test.ts restated against the oracle."""
import math

import numpy as np
import pytest

from caustic import camera_frame, furnace_scene, pack_scene
from caustic import _abi


def _opts(w, h, spp, bounces, rr, nee, seed):
    return _abi.ct_render_options(w, h, spp, bounces, int(rr), int(nee), seed)


@pytest.fixture(scope="module")
def furnace():
    sc = furnace_scene()
    return pack_scene(sc), camera_frame(sc.camera, 1.0).struct()


def test_furnace_naive(oracle, furnace):  # furnace.test.ts:28-43
    ps, frame = furnace
    img = oracle.render_image(ps, frame, _opts(8, 8, 4096, 64, False, False, 3))
    assert (np.abs(img - 5) / 5 < 0.05).all()
    # Without NEE and roulette every sample is the geometric series 5 (1 - 0.8^65).
    assert np.abs(img - 5 * (1 - 0.8 ** 65)).max() < 1e-4


def test_furnace_nee_mis(oracle, furnace):  # furnace.test.ts:45-63
    ps, frame = furnace
    assert len(ps.lights) == 1
    img = oracle.render_image(ps, frame, _opts(4, 4, 4096, 64, False, True, 9))
    assert abs(img.mean() - 5) / 5 < 0.03
    assert (np.abs(img - 5) / 5 < 0.08).all()


def test_furnace_roulette(oracle, furnace):  # furnace.test.ts:65-81
    ps, frame = furnace
    img = oracle.render_image(ps, frame, _opts(4, 4, 4096, 64, True, False, 5))
    assert abs(img.mean() - 5) / 5 < 0.03


# ---- materials.test.ts ----------------------------------------------------------
def _normalize(v):
    v = np.asarray(v, np.float64)
    return v / np.sqrt((v * v).sum())


def test_cosine_hemisphere_mean_and_histogram(oracle):  # materials.test.ts:21-63
    from caustic import Rng

    rng = Rng(42)
    n = _normalize([0.3, 0.8, -0.5])
    N = 100_000
    u = rng.draw(2 * N).reshape(N, 2)
    cos = np.empty(N)
    for i in range(N):
        d = oracle.vector(0, [*n, u[i, 0], u[i, 1]])[:3]
        assert abs(np.linalg.norm(d) - 1) < 1e-6
        cos[i] = d @ n
    assert (cos >= 0).all()
    assert abs(cos.mean() - 2 / 3) / (2 / 3) < 0.02
    hist = np.histogram(np.minimum(cos, 0.999999), bins=10, range=(0, 1))[0]
    lo = np.arange(10) / 10
    expected = ((lo + 0.1) ** 2 - lo ** 2) * N
    assert (np.abs(hist - expected) / expected < 0.08).all()


def test_dielectric_fresnel_and_tir(oracle):  # materials.test.ts:82-110
    r0 = ((1.5 - 1) / (1.5 + 1)) ** 2
    assert abs(oracle.scalar(3, 1, 1, 1.5) - r0) < 1e-6
    assert abs(oracle.scalar(4, 1, 1, 1.5) - r0) < 1e-6
    assert abs(oracle.scalar(3, 0, 1, 1.5) - 1) < 1e-6
    crit = math.asin(1 / 1.5)
    th = crit + 0.05
    assert oracle.scalar(4, math.cos(th), 1.5, 1) == 1
    d = _normalize([math.sin(th), -math.cos(th), 0])
    out = oracle.vector(3, [*d, 0, 1, 0, 1.5, 0, 0.999])
    assert out[3] == 1  # reflected
    from caustic import Rng

    rng = Rng(3)
    d = _normalize([0.5, -1, 0.2])
    R = oracle.scalar(4, -d[1], 1, 1.5)
    N = 20_000
    refl = sum(oracle.vector(3, [*d, 0, 1, 0, 1.5, 1, rng.next()])[3] for _ in range(N))
    assert abs(refl / N - R) < 0.01


def test_metal_mirror_and_fuzz(oracle):  # materials.test.ts:114-138
    d = _normalize([0.4, -0.7, 0.2])
    n = _normalize([0.1, 1, 0.05])
    r = oracle.vector(2, [*d, *n, 0, 0.1, 0.2, 0.3])[:3]
    expect = d - 2 * (d @ n) * n
    assert np.abs(r - expect).max() < 1e-12
    from caustic import Rng

    rng = Rng(5)
    s = 0.0
    for _ in range(1000):
        s += oracle.vector(2, [0, -1, 0, 0, 1, 0, 0.3, rng.next(), rng.next(), rng.next()])[1]
    assert s / 1000 > 0.9


def test_unit_vectors_and_power_heuristic(oracle):  # materials.test.ts:142-160
    from caustic import Rng

    rng = Rng(11)
    up = 0
    for _ in range(5000):
        v = oracle.vector(1, [rng.next(), rng.next()])[:3]
        assert abs(np.linalg.norm(v) - 1) < 1e-9
        up += v[2] > 0
    assert abs(up / 5000 - 0.5) < 0.03
    for a, b in ((0.3, 0.9), (2, 0.1), (1, 1)):
        assert abs(oracle.scalar(5, a, b) + oracle.scalar(5, b, a) - 1) < 1e-12
    assert oracle.scalar(5, 0, 0) == 0


def test_checker_parity(oracle):  # materials.ts:177-181
    assert oracle.vector(5, [0.1, 0.1, 0.1, 1])[0] == 1
    assert oracle.vector(5, [0.6, 0.1, 0.1, 1])[0] == 0
    assert oracle.vector(5, [-0.6, 0.1, 0.1, 1])[0] == 0
    assert oracle.vector(5, [-0.6, -0.6, 0.1, 1])[0] == 1

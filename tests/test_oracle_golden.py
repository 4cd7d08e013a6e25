"""Pins the oracle to the reference: its golden render and reference.test.ts.

tests/golden/cornell.ppm is the reference's own out/cornell.ppm
(renderCornellReference(96, 64, 16) with its defaults). The oracle must
reproduce it byte for byte; the qualitative checks of reference.test.ts and
the tone-mapping known points follow.
"""
import hashlib
import math
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def cornell(oracle):
    return oracle.cornell_reference(96, 64, 16)


def test_golden_fixture_intact():
    data = (GOLDEN / "cornell.ppm").read_bytes()
    want = (GOLDEN / "cornell.ppm.sha256").read_text().split()[0]
    assert hashlib.sha256(data).hexdigest() == want


def test_oracle_reproduces_reference_ppm_byte_exact(oracle, cornell):
    from caustic.tonemap import decode_ppm, encode_ppm

    linear, rgba = cornell
    w, h, ref_rgb = decode_ppm((GOLDEN / "cornell.ppm").read_bytes())
    assert (w, h) == (96, 64)
    mine = rgba.reshape(-1, 4)[:, :3].reshape(-1)
    assert np.array_equal(mine, ref_rgb), f"{int((mine != ref_rgb).sum())} bytes differ"
    assert encode_ppm(96, 64, rgba) == (GOLDEN / "cornell.ppm").read_bytes()


def test_oracle_result_independent_of_thread_count(oracle):
    a, _ = oracle.cornell_reference(96, 64, 4, nthreads=1)
    b, _ = oracle.cornell_reference(96, 64, 4, nthreads=5)
    assert np.array_equal(a, b)


def _px(linear, x, y, w=96):
    o = (y * w + x) * 3
    return linear[o:o + 3].astype(np.float64)


def test_finite_non_black(cornell):  # reference.test.ts:9-16
    linear, _ = cornell
    assert np.isfinite(linear).all()
    assert linear.sum() > 0


def test_center_brighter_than_corner(cornell):  # reference.test.ts:18-23
    linear, _ = cornell
    lum = lambda p: 0.2126 * p[0] + 0.7152 * p[1] + 0.0722 * p[2]
    assert lum(_px(linear, 48, 32)) > lum(_px(linear, 0, 63))


def test_red_and_green_walls(cornell):  # reference.test.ts:25-48
    linear, _ = cornell
    r = g = 0.0
    for y in range(24, 40):
        for x in range(1, 7):
            p = _px(linear, x, y)
            r, g = r + p[0], g + p[1]
    assert r > g * 1.5
    r = g = 0.0
    for y in range(24, 40):
        for x in range(89, 95):
            p = _px(linear, x, y)
            r, g = r + p[0], g + p[1]
    assert g > r * 1.5


def test_ppm_round_trip(cornell):  # reference.test.ts:50-58
    from caustic.tonemap import decode_ppm, encode_ppm

    _, rgba = cornell
    w, h, rgb = decode_ppm(encode_ppm(96, 64, rgba))
    assert (w, h) == (96, 64)
    o = (32 * 96 + 48)
    assert rgb[o * 3] == rgba[o * 4] and rgb[o * 3 + 1] == rgba[o * 4 + 1]


def test_tonemap_known_points(oracle):  # reference.test.ts:61-94
    prev_a = prev_r = -1.0
    for i in range(201):
        x = i * 0.1
        a, r = oracle.scalar(0, x), oracle.scalar(1, x)
        assert a >= prev_a - 1e-9 and r >= prev_r - 1e-9
        assert a <= 1 and r < 1
        prev_a, prev_r = a, r
    assert oracle.scalar(0, 0) == 0 and oracle.scalar(1, 0) == 0
    assert abs(oracle.scalar(1, 1) - 0.5) < 1e-12
    assert oracle.scalar(2, 0) == 0 and oracle.scalar(2, 1) == 1
    assert abs(oracle.scalar(2, 0.5) - 0.7354) < 1e-3
    accum = np.array([2, 2, 2], np.float32)
    a = oracle.tonemap(accum, 1, 1, 4, 0, aces=False)
    want = math.floor(oracle.scalar(2, oracle.scalar(1, 0.5)) * 255 + 0.5)
    assert a[0] == want and a[3] == 255
    b = oracle.tonemap(accum, 1, 1, 4, 1, aces=False)
    assert b[0] == math.floor(oracle.scalar(2, oracle.scalar(1, 1.0)) * 255 + 0.5)


def test_host_tonemap_matches_oracle(oracle, cornell):
    from caustic.tonemap import tonemap_buffer

    linear, rgba = cornell
    assert np.array_equal(tonemap_buffer(linear, 96, 64, 1, 0.0, "aces"), rgba)
    rng = np.random.default_rng(3)
    acc = (rng.random(300) * 8).astype(np.float32)
    for ev, mode in ((0.0, "aces"), (1.5, "reinhard"), (-2.0, "aces")):
        mine = tonemap_buffer(acc, 10, 10, 3, ev, mode)
        assert np.array_equal(mine, oracle.tonemap(acc, 10, 10, 3, ev, mode == "aces"))

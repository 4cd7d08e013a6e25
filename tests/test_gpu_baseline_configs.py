"""Parity at the benchmarked configurations themselves, at the sizes the bench times.

* Cornell unit box, 512 x 512, 16 spp, 8 bounces, NEE on, Russian roulette
  off, seed 1 (the headline render): per-pixel means within 3 combined
  standard errors of the oracle's (at most 1 % of channels outside), and each
  channel's image mean within 3 standard errors of the oracle's image mean,
  through the whole-path kernel and through the wavefront kernels.
* Traversal: the 1,000,000-triangle soup and all 16,777,216 rays of the
  benchmark: hit primitive ids equal the oracle's ordered walk
  (intersect.ts:202-282) except at verified ties within 1e-5 relative t, t
  within 4e-6 relative, misses exact. The skip-link walk
  (intersect.ts:290-365) is checked on the first 4 Mi rays.
* Caustic scene at its full icosphere level 7 (327,680 triangles), 480 x
  270, 16 spp, 12 bounces, Russian roulette on: 3 sigma.

The reference tests these follow: bvh.test.ts:88-146 (ids against brute
force), furnace.test.ts:28-81 and reference.test.ts:9-48 (image checks).
"""

import numpy as np
import pytest

import caustic as ct
from bench import CAUSTIC, CORNELL, TRAVERSAL
from test_gpu_render import gpu_sums, oracle_sums, three_sigma
from test_gpu_trace import check_closest

pytestmark = pytest.mark.gpu

CT_OPT_PATH_KERNEL = 4  # include/caustic.h


def image_mean_sigma(gpu, ora, spp):
    """Per channel: |GPU image mean - oracle image mean| in combined standard errors of the image mean."""
    (gs, gq), (os_, oq) = gpu, ora
    out = []
    for c in range(3):
        g, gq_c, o, oq_c = gs[c::3] / spp, gq[c::3] / spp, os_[c::3] / spp, oq[c::3] / spp
        n = len(g)
        var = (np.maximum(gq_c - g * g, 0) + np.maximum(oq_c - o * o, 0)).sum() / spp
        se = np.sqrt(var) / n
        out.append(abs(g.mean() - o.mean()) / max(se, 1e-12))
    return np.array(out)


@pytest.fixture(scope="module")
def cornell512(oracle, native_lib):
    sc = ct.cornell_unit_box()
    w, h, spp = CORNELL["width"], CORNELL["height"], CORNELL["spp"]
    packed = ct.pack_scene(sc)
    frame = ct.camera_frame(sc.camera, w / h)
    ora = oracle_sums(oracle, packed, frame, w, h, spp, CORNELL["seed"], CORNELL["max_bounces"],
                      CORNELL["russian_roulette"], CORNELL["nee"])
    return packed, frame, ora


@pytest.mark.parametrize("path_kernel", [1, 0], ids=["whole_path", "wavefront"])
def test_cornell_512_headline_three_sigma(cornell512, path_kernel):
    packed, frame, ora = cornell512
    w, h, spp = CORNELL["width"], CORNELL["height"], CORNELL["spp"]
    assert packed.prim_count <= 32  # the whole-path kernel's case
    with ct.DeviceScene(packed) as dev:
        ct._native.check(dev._lib.ct_scene_set_option(dev.handle, CT_OPT_PATH_KERNEL, path_kernel))
        gpu = gpu_sums(dev, frame, w, h, spp, CORNELL["seed"], CORNELL["max_bounces"], CORNELL["russian_roulette"],
                       CORNELL["nee"])
    frac_bad, gm, om = three_sigma(gpu, ora, spp)
    assert frac_bad <= 0.01, f"{frac_bad:.4f} of pixel channels outside 3 standard errors"
    sig = image_mean_sigma(gpu, ora, spp)
    assert (sig < 3).all(), f"image mean off by {sig} standard errors"
    assert np.isfinite(gm).all() and gm.mean() > 0


def test_cornell_512_render_image_equals_sums(cornell512):
    """renderImage (ct_render_image) at the headline size equals the summed passes / spp."""
    packed, frame, ora = cornell512
    w, h, spp = CORNELL["width"], CORNELL["height"], CORNELL["spp"]
    opts = ct.RenderOptions(max_bounces=CORNELL["max_bounces"], russian_roulette=CORNELL["russian_roulette"],
                            nee=CORNELL["nee"], width=w, height=h, spp=spp, seed=CORNELL["seed"])
    with ct.DeviceScene(packed) as dev:
        img = ct.render_image(dev, frame, opts)
        sums, _ = gpu_sums(dev, frame, w, h, spp, CORNELL["seed"], CORNELL["max_bounces"],
                           CORNELL["russian_roulette"], CORNELL["nee"])
    assert np.array_equal(img, (sums / spp).astype(np.float32))  # 1/16 is exact in float32


@pytest.fixture(scope="module")
def soup1m(native_lib):
    packed = ct.pack_scene(ct.triangle_soup(TRAVERSAL["triangles"], seed=TRAVERSAL["scene_seed"]))
    rays = ct.soup_rays(TRAVERSAL["rays"], seed=TRAVERSAL["ray_seed"])
    return packed, rays


def test_traversal_1m_soup_all_bench_rays(oracle, soup1m):
    packed, rays = soup1m
    with ct.DeviceScene(packed) as dev:
        hits = ct.intersect_closest(dev, rays)
    ties, n_hit = check_closest(oracle, packed, rays, hits, "soup1M")
    assert n_hit > 0.5 * len(rays)
    assert ties <= 1e-4 * len(rays)


def test_traversal_1m_soup_stackless(oracle, soup1m):
    packed, rays = soup1m
    rays = rays[: 1 << 22]
    prev = ct.set_traversal("stackless")
    try:
        with ct.DeviceScene(packed) as dev:
            hits = ct.intersect_closest(dev, rays)
    finally:
        ct.set_traversal(prev)
    ties, n_hit = check_closest(oracle, packed, rays, hits, "soup1M stackless")
    assert n_hit > 0.5 * len(rays)


def test_caustic_level7_three_sigma(oracle, native_lib):
    sc = ct.caustic_scene(level=7)
    packed = ct.pack_scene(sc)
    assert packed.prim_count > 327_680
    w, h, spp = 480, 270, 16
    frame = ct.camera_frame(sc.camera, w / h)
    with ct.DeviceScene(packed) as dev:
        gpu = gpu_sums(dev, frame, w, h, spp, CAUSTIC["seed"], CAUSTIC["max_bounces"], CAUSTIC["russian_roulette"],
                       CAUSTIC["nee"])
    ora = oracle_sums(oracle, packed, frame, w, h, spp, CAUSTIC["seed"], CAUSTIC["max_bounces"],
                      CAUSTIC["russian_roulette"], CAUSTIC["nee"])
    frac_bad, gm, om = three_sigma(gpu, ora, spp)
    assert frac_bad <= 0.01, f"{frac_bad:.4f} of pixel channels outside 3 standard errors"
    sig = image_mean_sigma(gpu, ora, spp)
    assert (sig < 3).all(), f"image mean off by {sig} standard errors"

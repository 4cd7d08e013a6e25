"""Batched rendering (ct_batch_*): every job's image equals the single-scene
render with the same frame indices, whatever the wave packing, and the
graph replays accumulate further passes correctly."""
import numpy as np
import pytest

import caustic as ct
from caustic import _native

pytestmark = pytest.mark.gpu


def _jobs(scenes, spp=3):
    jobs = []
    for i, (sc, w, h) in enumerate(scenes):
        dev = ct.DeviceScene.from_scene(sc)
        jobs.append(ct.Job(dev, ct.camera_frame(sc.camera, w / h), w, h, spp, seed=i + 1))
    return jobs


PER_JOB = 3  # ct_batch_info walk: every job walks as its scene does alone


def _force_walk(scene, walk):
    # Same trace walk as the batch: in float32, walks that visit nodes in a
    # different order can break exact ties (a quad's shared diagonal) the
    # other way, which changes a path but not the estimator. A per-job batch
    # needs no override (-1 keeps the scene's own choice).
    from caustic import _native

    _native.check(scene._lib.ct_scene_set_option(scene.handle, 1, -1 if walk == PER_JOB else walk))


def _single(job, opts, walk):
    _force_walk(job.scene, walk)
    return ct.render_image(job.scene, job.frame, ct.RenderOptions(
        max_bounces=opts.max_bounces, russian_roulette=opts.russian_roulette, nee=opts.nee,
        width=job.width, height=job.height, spp=job.spp, seed=job.seed))


@pytest.fixture(scope="module")
def scenes(native_lib):
    out = [(ct.batch_scene(11, 2_000, 3), 48, 48), (ct.batch_scene(12, 20_000, 0), 32, 24),
           (ct.cornell_unit_box(), 40, 40), (ct.caustic_scene(level=3), 36, 20), (ct.CORNELL_BOX, 24, 16),
           (ct.batch_scene(13, 5_000, 12), 17, 9)]
    return out


@pytest.mark.parametrize("wave_paths,walk", [(0, -1), (1000, -1), (777, 0), (5000, 2), (3000, 1)])
def test_batch_equals_single_renders(scenes, wave_paths, walk):
    opts = ct.TraceOptions(max_bounces=8, russian_roulette=True, nee=True)
    jobs = _jobs(scenes)
    with ct.BatchRenderer(jobs, opts, wave_paths=wave_paths, walk=walk) as br:
        br.run()
        imgs = br.images()
        info = br.info()
        if wave_paths:
            assert info["waves"] > 3
        for job, img in zip(jobs, imgs):
            want = _single(job, opts, info["walk"])
            assert np.isfinite(img).all()
            assert np.array_equal(img, want), job.scene.packed.prim_count
        # a second run of the same graph adds the same passes again
        br.run()
        for img, again in zip(imgs, br.images()):
            assert np.allclose(again, 2 * img, rtol=1e-5, atol=1e-6)
    for j in jobs:
        j.scene.close()


def test_batch_progressive_frames(scenes):
    """Replaying with new first frames renders the next passes (progressive refinement)."""
    opts = ct.TraceOptions(max_bounces=6, russian_roulette=False, nee=True)
    jobs = _jobs(scenes[:3], spp=2)
    with ct.BatchRenderer(jobs, opts, wave_paths=900) as br:
        br.run()
        br.set_first_frames([j.seed * 7919 + 2 for j in jobs])
        br.run()
        got = br.images()
        walk = br.info()["walk"]
        assert walk == PER_JOB

    for job, img in zip(jobs, got):
        _force_walk(job.scene, walk)
        four = ct.render_image(job.scene, job.frame, ct.RenderOptions(
            max_bounces=6, russian_roulette=False, nee=True, width=job.width, height=job.height, spp=4,
            seed=job.seed))
        assert np.allclose(img / 2, four, rtol=1e-5, atol=1e-6)
        job.scene.close()


def test_batch_rejects_bad_jobs(scenes):
    opts = ct.TraceOptions()
    jobs = _jobs(scenes[:1])
    for walk in (3, -2):
        with pytest.raises(ct.CausticError, match="batch walk"):
            ct.BatchRenderer(jobs, opts, walk=walk)
    bad = [ct.Job(jobs[0].scene, jobs[0].frame, 0, 8, 1)]
    with pytest.raises(ct.CausticError):
        ct.BatchRenderer(bad, opts)
    with pytest.raises(ct.CausticError, match="wave_paths"):
        ct.BatchRenderer(jobs, opts, wave_paths=-1)
    jobs[0].scene.close()


def _lens_box():
    import dataclasses

    return dataclasses.replace(ct.cornell_unit_box(), camera=ct.camera_at((0, 0.5, 1.6), (0, 0.5, 0), 32, 0.04, 1.55))


def _sky_box():
    import dataclasses

    return dataclasses.replace(ct.cornell_unit_box(), sky=ct.SkyGradient((0.35, 0.55, 0.95), (1.0, 0.95, 0.85), 1.5))


@pytest.mark.parametrize("scene_fn", [ct.cornell_unit_box, lambda: ct.CORNELL_BOX, _lens_box, _sky_box])
def test_path_kernel_equals_wavefront(native_lib, scene_fn):
    """A scene of at most 32 primitives renders alone through the whole-path
    kernel (k_paths) and in a batch through the wavefront kernels: the images
    are equal bit for bit, with and without Russian roulette and NEE, through
    a pinhole and a thin lens, under no sky and a gradient sky."""
    scene = ct.DeviceScene.from_scene(scene_fn())
    assert scene.walk == 2 and scene.packed.prim_count <= 32
    frame = ct.camera_frame(scene_fn().camera, 40 / 30)
    for rr, nee in [(False, True), (True, True), (True, False)]:
        opts = ct.TraceOptions(max_bounces=8, russian_roulette=rr, nee=nee)
        alone = ct.render_image(scene, frame, ct.RenderOptions(max_bounces=8, russian_roulette=rr, nee=nee,
                                                               width=40, height=30, spp=9, seed=5))
        with ct.BatchRenderer([ct.Job(scene, frame, 40, 30, 9, seed=5)], opts) as br:
            br.run()
            batch = br.images()[0]
        assert np.array_equal(alone.reshape(-1), batch.reshape(-1)), (rr, nee)
        # the same scene alone with the whole-path kernel switched off (CT_OPT_PATH_KERNEL = 0)
        _native.check(scene._lib.ct_scene_set_option(scene.handle, 4, 0))
        wave = ct.render_image(scene, frame, ct.RenderOptions(max_bounces=8, russian_roulette=rr, nee=nee,
                                                              width=40, height=30, spp=9, seed=5))
        _native.check(scene._lib.ct_scene_set_option(scene.handle, 4, 1))
        assert np.array_equal(alone.reshape(-1), wave.reshape(-1)), (rr, nee)
    scene.close()

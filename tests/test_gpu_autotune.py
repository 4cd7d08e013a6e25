"""The integrator's autotuner on the device: it measures the candidates,
applies the fastest, stores and reuses its table, and its choices change
render time only, never the image."""
import ctypes as C

import numpy as np
import pytest

import caustic as ct
from caustic import autotune as at

pytestmark = pytest.mark.gpu


def _render(dev, frame, opts):
    return ct.render_image(dev, frame, opts).reshape(-1)


def test_autotune_applies_best_and_reuses_table(native_lib, tmp_path):
    scene = ct.batch_scene(31, 3_000, 6)
    opts = ct.RenderOptions(max_bounces=4, russian_roulette=True, nee=True, width=40, height=32, spp=2, seed=3)
    frame = ct.camera_frame(scene.camera, 40 / 32)
    table = tmp_path / "tune.json"
    with ct.DeviceScene.from_scene(scene) as dev:
        res = at.autotune(dev, frame, opts, table_path=table, reps=1, probe_spp=1)
        pairs = at.candidates(dev, opts)
        assert len(res.measured) == len(pairs) + len(at.BLOCK_CANDIDATES)
        assert res.best in res.measured and res.best.ms == min(c.ms for c in res.measured)
        assert all(c.ms > 0 for c in res.measured)
        assert dev.walk == res.best.walk
        assert table.exists()
    with ct.DeviceScene.from_scene(scene) as dev:
        again = at.autotune(dev, frame, opts, table_path=table, reps=1, probe_spp=1)
        assert again.key == res.key and again.best == res.best  # read from the table, not re-measured
        assert again.measured == res.measured
        assert dev.walk == res.best.walk


@pytest.mark.parametrize("scene_fn", [lambda: ct.batch_scene(32, 4_000, 3), ct.cornell_unit_box])
def test_trace_blocks_change_timing_only(native_lib, scene_fn):
    """Fewer resident blocks per SM for the trace (or whole-path) launches
    give the same image bit for bit."""
    scene = scene_fn()
    opts = ct.RenderOptions(max_bounces=6, russian_roulette=True, nee=True, width=48, height=40, spp=5, seed=11)
    frame = ct.camera_frame(scene.camera, 48 / 40)
    with ct.DeviceScene.from_scene(scene) as dev:
        want = _render(dev, frame, opts)
        for blocks in (1, 3):
            at.apply(dev, at.Choice(dev.walk, 0, 0.0, blocks))
            assert np.array_equal(_render(dev, frame, opts), want), blocks
        lib = dev._lib
        assert lib.ct_scene_set_option(dev.handle, at.OPT_TRACE_BLOCKS, C.c_int64(65)) != 0

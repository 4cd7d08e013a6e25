"""Host logic of the autotuner, without a GPU: candidate sets, table keys,
the JSON table (older tables without the launch-shape field included), and
reuse of a stored choice without measuring."""
import json

import pytest

import caustic as ct
from caustic import autotune as at


class _FakeScene:
    """What the tuner reads of a DeviceScene when it does not measure."""

    def __init__(self, packed):
        self.packed = packed
        self.applied = []


@pytest.fixture(scope="module")
def fake(native_lib):
    return _FakeScene(ct.pack_scene(ct.batch_scene(41, 3_000, 2)))


def _opts(w=64, h=48, spp=4):
    return ct.RenderOptions(max_bounces=6, russian_roulette=True, nee=True, width=w, height=h, spp=spp, seed=1)


def test_candidates_cover_walks_and_waves(fake):
    cands = at.candidates(fake, _opts())
    walks = sorted({w for w, _ in cands})
    waves = sorted({v for _, v in cands})
    assert walks == [0, 1, 2]
    assert waves[0] == 0 and all(v >= 64 * 48 for v in waves[1:])
    assert len(cands) == len(walks) * len(waves)
    # a render larger than every fixed wave size keeps only the library default
    assert {v for _, v in at.candidates(fake, _opts(w=4096, h=4096))} == {0}


def test_key_names_scene_shape_and_render(fake):
    k1, k2 = at.scene_key(fake, _opts()), at.scene_key(fake, _opts(spp=8))
    assert k1 != k2 and k1.startswith(f"prims={fake.packed.prim_count}:nodes={fake.packed.node_count}:")
    assert at.scene_key(fake, _opts(w=60, h=50)) == k1  # same power-of-two pixel bucket


def test_table_round_trip_and_older_entries(tmp_path):
    path = tmp_path / "tune.json"
    best = at.Choice(1, 1 << 22, 3.5, 6)
    at._store(path, {"k": {"best": best.__dict__, "measured": [best.__dict__]}})
    back = at._load(path)
    assert at.Choice(**back["k"]["best"]) == best
    old = {"walk": 0, "wave_paths": 0, "ms": 2.0}  # a table written before the launch-shape stage
    assert at.Choice(**old).blocks == 0


def test_stored_choice_is_reused_without_measuring(fake, tmp_path, monkeypatch):
    opts = _opts()
    key = at.scene_key(fake, opts)
    best = at.Choice(2, 0, 1.25, 4)
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({key: {"best": best.__dict__, "measured": [best.__dict__]}}))
    monkeypatch.setattr(at, "_time_render", lambda *a, **k: pytest.fail("measured although the table has the key"))
    monkeypatch.setattr(at, "apply", lambda dev, choice: dev.applied.append(choice))
    res = at.autotune(fake, None, opts, table_path=path)
    assert res.best == best and fake.applied[-1] == best and res.key == key

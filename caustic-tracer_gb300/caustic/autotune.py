"""Autotuner for the integrator's launch choices.

For a scene and a render size it times every admissible pair of
(trace walk form, paths per wave) on a short render, then, for the fastest
pair, the launch shape of the trace kernels (resident 128-thread blocks per
SM: as many as fit, or 8, 6 or 4), applies the fastest choice to the scene
(ct_scene_set_option) and records the measurements in a JSON table keyed by
the scene's shape (primitive and node counts, tree depth) and the render
size, so later renders of similar work reuse the choice without
re-measuring. Walk forms: 0 ordered walk per thread, 1 ordered walk with
persistent lane refill, 2 stackless skip-link walk. None of the choices
changes an image, only the time it takes.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import pathlib
import threading
from dataclasses import asdict, dataclass, field
from typing import Dict, List, Optional, Tuple

from . import _abi, _native
from .camera import CameraFrame
from .tracer import DeviceScene, RenderOptions

OPT_WALK = 1
OPT_WAVE_PATHS = 2
OPT_TRACE_BLOCKS = 3
BLOCK_CANDIDATES = (8, 6, 4)  # blocks per SM tried besides "as many as fit" (0)
WALK_NAMES = {0: "ordered/thread", 1: "ordered/persistent", 2: "skip-link"}
_lock = threading.Lock()


@dataclass
class Choice:
    walk: int
    wave_paths: int
    ms: float
    blocks: int = 0  # trace blocks per SM (0: as many as fit)


@dataclass
class TuneResult:
    key: str
    best: Choice
    measured: List[Choice] = field(default_factory=list)


def scene_key(dev: DeviceScene, opts: RenderOptions) -> str:
    p = dev.packed
    depth = _tree_depth(p.nodes, p.node_count)
    size = 1 << max(0, (opts.width * opts.height - 1).bit_length())  # power-of-two pixel bucket
    return f"prims={p.prim_count}:nodes={p.node_count}:depth={depth}:pixels<={size}:spp={opts.spp}:bounces={opts.max_bounces}"


def _tree_depth(nodes, count: int) -> int:
    if count == 0:
        return 0
    depth, stack = 0, [(0, 1)]
    while stack:
        i, d = stack.pop()
        depth = max(depth, d)
        if nodes[i * 8 + 7] < 0:
            left = i + 1
            stack.append((left, d + 1))
            stack.append((int(nodes[left * 8 + 3]), d + 1))
    return depth


def _time_render(dev: DeviceScene, frame: CameraFrame, opts: RenderOptions, reps: int) -> float:
    out = __import__("numpy").empty(opts.width * opts.height * 3, "float32")
    f, o = frame.struct(), opts.struct()
    stats = _abi.ct_stats()
    best = float("inf")
    for _ in range(reps + 1):  # first call warms caches and allocations
        _native.check(dev._lib.ct_render_image(dev.handle, C.byref(f), C.byref(o), _native.ptr(out), C.byref(stats)))
        best = min(best, stats.kernel_ms)
    return best


def candidates(dev: DeviceScene, opts: RenderOptions) -> List[Tuple[int, int]]:
    depth = _tree_depth(dev.packed.nodes, dev.packed.node_count)
    walks = [2] + ([0, 1] if depth <= 64 else [])
    pixels = opts.width * opts.height
    waves = sorted({0, *(w for w in (1 << 21, 1 << 22, 1 << 23) if w >= pixels)})
    return [(wk, wv) for wk in walks for wv in waves]


def autotune(dev: DeviceScene, frame: CameraFrame, opts: RenderOptions, table_path: Optional[os.PathLike] = None,
             reps: int = 2, probe_spp: int = 2) -> TuneResult:
    """Measures the candidates on a `probe_spp`-sample render and applies the fastest."""
    key = scene_key(dev, opts)
    table = _load(table_path)
    if key in table:
        best = Choice(**table[key]["best"])
        apply(dev, best)
        return TuneResult(key, best, [Choice(**c) for c in table[key]["measured"]])
    probe = RenderOptions(max_bounces=opts.max_bounces, russian_roulette=opts.russian_roulette, nee=opts.nee,
                          width=opts.width, height=opts.height, spp=min(opts.spp, probe_spp), seed=opts.seed)
    measured = []
    for walk, wave in candidates(dev, opts):
        try:
            apply(dev, Choice(walk, wave, 0.0))
        except _native.CausticError:  # e.g. an ordered walk whose stack this tree could outgrow
            continue
        measured.append(Choice(walk, wave, _time_render(dev, frame, probe, reps)))
    best = min(measured, key=lambda c: c.ms)
    for blocks in BLOCK_CANDIDATES:  # launch shape of the best pair
        apply(dev, Choice(best.walk, best.wave_paths, 0.0, blocks))
        measured.append(Choice(best.walk, best.wave_paths, _time_render(dev, frame, probe, reps), blocks))
    best = min(measured, key=lambda c: c.ms)
    apply(dev, best)
    if table_path is not None:
        table[key] = {"best": asdict(best), "measured": [asdict(c) for c in measured]}
        _store(table_path, table)
    return TuneResult(key, best, measured)


def apply(dev: DeviceScene, choice: Choice) -> None:
    _native.check(dev._lib.ct_scene_set_option(dev.handle, OPT_WALK, int(choice.walk)))
    _native.check(dev._lib.ct_scene_set_option(dev.handle, OPT_WAVE_PATHS, int(choice.wave_paths)))
    _native.check(dev._lib.ct_scene_set_option(dev.handle, OPT_TRACE_BLOCKS, int(choice.blocks)))


def _load(path) -> Dict:
    if path is None or not pathlib.Path(path).exists():
        return {}
    with _lock:
        return json.loads(pathlib.Path(path).read_text())


def _store(path, table: Dict) -> None:
    with _lock:
        p = pathlib.Path(path)
        tmp = p.with_suffix(p.suffix + ".tmp")
        tmp.write_text(json.dumps(table, indent=1, sort_keys=True))
        os.replace(tmp, p)

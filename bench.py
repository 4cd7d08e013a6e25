"""Benchmark of the GB300 path tracer (one JSON line on rank 0).

Workloads
  cornell   (default) Cornell box, 512 x 512, 16 spp, 8 bounces, NEE on,
            Russian roulette off, seed 1. A step is one renderImage
            (4,194,304 samples). Metric: Msamples/s.
  traversal 1,000,000-triangle soup, 16,777,216 rays; a step is one
            intersectClosest batch over all rays. Metric: Mrays/s.
  caustic   glass icosphere (327,680 triangles) among 64 spheres,
            1920 x 1080, 64 spp, 12 bounces, Russian roulette on.
  batched   256 scenes rendered by one CUDA graph, against the same jobs as
            consecutive plain renders.
  served    a request trace through the continuous-batching server, against
            one plain renderImage per request (throughput all queued at
            once; p50/p99 latency under Poisson arrivals).
  display   tonemapBuffer of a 3840 x 2160 sum buffer into RGBA8 on the
            device (ct_tonemap_device). Metric: Mpixels/s.

The default line (cornell) also carries the traversal and caustic workloads
as sub-records, each with its own value, roofline, CPU baseline and e2e, and
the batched and served forms (5 and 2 timed steps) with their plain
baselines.

`value` is device time with inputs resident in HBM (CUDA events on the
launching stream, max over ranks); `e2e` is the same metric through the
C-ABI host-pointer call, host<->device copies included. Each rank renders
its own samples (different frame indices / ray seeds): weak scaling, no
data-path collective.

--impl reference times the reference's CPU algorithm (the C++ restatement in
oracle/, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
for _p in (ROOT / "caustic-tracer_gb300", ROOT / "tests"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

CORNELL = dict(width=512, height=512, spp=16, max_bounces=8, russian_roulette=False, nee=True, seed=1)
CAUSTIC = dict(width=1920, height=1080, spp=64, max_bounces=12, russian_roulette=True, nee=True, seed=1)
TRAVERSAL = dict(triangles=1_000_000, rays=16_777_216, scene_seed=2024, ray_seed=77)
DISPLAY = dict(width=3840, height=2160, samples=64, exposure_ev=0.0, mode="aces", seed=11)
SIZE_OVERRIDE = None  # (width, height, spp) of a render workload, for profiling captures
# Paths a render needs to fill the GPU through its bounces: 152 SMs x 1,536
# resident lanes of the trace kernels = 233,472, times 4 for the tail of later
# bounces, where paths have ended.
FILL_PATHS = 1 << 20
RAY_BYTES, HIT_BYTES, BOX_BYTES, TRI_BYTES, SPHERE_BYTES = 32, 16, 32, 48, 32
ACCUM_BYTES_PER_SAMPLE = 12


CT_OPT_PATH_KERNEL = 4  # include/caustic.h

def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["cornell", "traversal", "caustic", "batched", "served", "display"], default="cornell")
    ap.add_argument("--jobs", type=int, default=256, help="batched: number of scenes")
    ap.add_argument("--requests", type=int, default=128, help="served: number of requests")
    ap.add_argument("--trace", choices=["c5", "preview"], default="c5",
                    help="served: the request mix (c5: 128-1024 squared, 1-256 spp; preview: 128-256 squared, "
                         "1-8 spp)")
    ap.add_argument("--small", action="store_true", help="reduced sizes for profiling captures")
    ap.add_argument("--rays", type=int, default=0, help="traversal: trace only this many rays (profiling)")
    ap.add_argument("--size", default="", help="cornell/caustic: WxHxSPP instead of the configuration's (profiling)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="cornell: leave out the traversal and caustic sub-records of the default line")
    ap.add_argument("--cpu-seconds", type=float, default=8.0,
                    help="--impl reference: seconds of oracle work in the calibration run (a step is a quarter)")
    return ap.parse_args()


# ---- clocks ------------------------------------------------------------------------
class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.samples = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---- helpers -----------------------------------------------------------------------
def peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_record(workload: str):
    path = ROOT / "profiles" / "traffic.json"
    if path.exists():
        return json.loads(path.read_text()).get(workload)
    return None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---- workloads --------------------------------------------------------------------
_SCENES: dict = {}
_RAYS: dict = {}


class OracleStream:
    """Scene generators draw from the oracle's restatement of Rng inside this
    block, so a process that times the reference algorithm never loads the
    CUDA library (the draws are the same numbers either way)."""

    def __enter__(self):
        import caustic.rng as rng
        import oracle_lib as oracle

        self.prev = rng.set_stream(oracle.rng_stream_state)
        return self

    def __exit__(self, *exc):
        import caustic.rng as rng

        rng.set_stream(self.prev)


def _pack(scene, oracle_pack: bool):
    """packScene through the library's packer, or the oracle's (the reference arm)."""
    if oracle_pack:
        import oracle_lib as oracle

        return oracle.pack(scene)
    import caustic as ct

    return ct.pack_scene(scene)


def traversal_inputs(rank: int, small: bool, rays: int = 0, oracle_pack: bool = False):
    """The 1,000,000-triangle soup (packed) and the 16,777,216 query rays (cached per process)."""
    import contextlib

    import caustic as ct

    tris = 100_000 if small else TRAVERSAL["triangles"]
    nrays = rays or ((1 << 20) if small else TRAVERSAL["rays"])
    ctx = OracleStream() if oracle_pack else contextlib.nullcontext()
    key = ("traversal", small, oracle_pack)
    with ctx:
        if key not in _SCENES:
            _SCENES[key] = _pack(ct.triangle_soup(tris, seed=TRAVERSAL["scene_seed"]), oracle_pack)
        rkey = (rank, nrays)
        if rkey not in _RAYS:
            _RAYS[rkey] = ct.soup_rays(nrays, seed=TRAVERSAL["ray_seed"] + rank)
    return _SCENES[key], _RAYS[rkey]


def render_cfg(workload: str, small: bool) -> dict:
    if workload == "display":
        cfg = dict(DISPLAY)
        if small:
            cfg.update(width=1920, height=1080)
        return cfg
    if workload == "caustic":
        cfg = dict(CAUSTIC)
        if small:
            cfg.update(width=480, height=270, spp=4)
    else:
        cfg = dict(CORNELL)
        if small:
            cfg.update(width=128, height=128, spp=4)
    if SIZE_OVERRIDE:
        cfg.update(width=SIZE_OVERRIDE[0], height=SIZE_OVERRIDE[1], spp=SIZE_OVERRIDE[2])
    return cfg


def display_inputs(small: bool):
    """A seeded synthetic sum buffer (width*height*3 float32) for the display
    workload: per-channel radiance log-normal around 0.37 (sigma 1.5) times
    the sample count, so both tone curves and their clamps are exercised."""
    key = ("display", small)
    if key not in _SCENES:
        cfg = render_cfg("display", small)
        rng = np.random.default_rng(cfg["seed"])
        n = cfg["width"] * cfg["height"] * 3
        _SCENES[key] = (rng.lognormal(-1.0, 1.5, n) * cfg["samples"]).astype(np.float32)
    return _SCENES[key], render_cfg("display", small)


def render_inputs(workload: str, small: bool, oracle_pack: bool = False):
    """Packed scene, camera frame and render options of a render workload (cached per process)."""
    import contextlib

    import caustic as ct

    cfg = render_cfg(workload, small)
    key = (workload, small, oracle_pack)
    if key not in _SCENES:
        with OracleStream() if oracle_pack else contextlib.nullcontext():
            scene = ct.caustic_scene(level=5 if small else 7) if workload == "caustic" else ct.cornell_unit_box()
            _SCENES[key] = (_pack(scene, oracle_pack), ct.camera_frame(scene.camera, cfg["width"] / cfg["height"]))
    packed, frame = _SCENES[key]
    return packed, frame, cfg


def cpu_reference(workload: str, small: bool, target_s: float = 12.0):
    """Times the oracle (the reference algorithm in C++, scenes packed by the
    oracle's own packScene) on a bounded sample; returns a dict."""
    import oracle_lib as oracle
    from caustic import _abi

    threads = os.cpu_count() or 1
    if workload == "traversal":
        packed, rays = traversal_inputs(0, small, oracle_pack=True)
        n = 1 << 14
        while True:
            t0 = time.perf_counter()
            _, _, _, _, cnt = oracle.trace(packed, rays[:n], 0, nthreads=threads)
            dt = time.perf_counter() - t0
            if dt >= target_s / 4 or n >= len(rays):
                break
            n = min(len(rays), int(n * max(2.0, min(8.0, target_s / 4 / max(dt, 1e-3)))))
        bpr = RAY_BYTES + HIT_BYTES + (BOX_BYTES * cnt[0] + TRI_BYTES * cnt[1] + SPHERE_BYTES * cnt[2]) / n
        return {"value": n / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                "sample": f"first {n} of the {len(rays)} rays, ordered walk (intersectClosest), {threads} threads",
                "bytes_per_unit": bpr, "counts_per_ray": {"aabb": cnt[0] / n, "tri": cnt[1] / n, "sphere": cnt[2] / n},
                "seconds": dt}
    if workload == "display":
        sums, cfg = display_inputs(small)
        w, h = cfg["width"], cfg["height"]
        rows = 16
        while True:
            t0 = time.perf_counter()
            oracle.tonemap(sums[: w * rows * 3], w, rows, cfg["samples"], cfg["exposure_ev"])
            dt = time.perf_counter() - t0
            if dt >= target_s / 8 or rows >= h:
                break
            rows = min(h, int(rows * max(2.0, min(8.0, target_s / 8 / max(dt, 1e-3)))))
        return {"value": w * rows / dt / 1e6, "unit": "Mpixels/s", "cores": 1, "kind": "port",
                "sample": f"{w}x{rows} pixels of the {w}x{h} sum buffer, tonemapBuffer (ACES), 1 thread",
                "seconds": dt, "bytes_per_unit": 16}
    packed, frame, cfg = render_inputs(workload, small, oracle_pack=True)

    # Rows of the image at full spp until the sample takes long enough.
    w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
    rows = 4
    while True:
        opts = _abi.ct_render_options(w, rows, spp, cfg["max_bounces"], int(cfg["russian_roulette"]),
                                      int(cfg["nee"]), cfg["seed"])
        fs = frame.struct()
        t0 = time.perf_counter()
        oracle.render_image(packed, fs, opts, nthreads=threads)
        dt = time.perf_counter() - t0
        if dt >= target_s / 4 or rows >= h:
            break
        rows = min(h, int(rows * max(2.0, min(8.0, target_s / 4 / max(dt, 1e-3)))))
    samples = w * rows * spp
    work = cornell_work_counts(packed, frame, cfg)
    return {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{w}x{rows} pixels x {spp} spp of the {w}x{h} render, {threads} threads",
            "seconds": dt, "work_per_sample": work}


def cornell_work_counts(packed, frame, cfg, npix: int = 8192):
    """Mean work per sample of the reference algorithm (oracle) over a pixel subsample:
    closest rays, shadow rays, and the box/triangle/sphere tests of each query kind."""
    import oracle_lib as oracle
    from caustic import _abi

    topts = _abi.ct_trace_options(cfg["max_bounces"], int(cfg["russian_roulette"]), int(cfg["nee"]))
    fs = frame.struct()
    tot = np.zeros(10)
    pixels = cfg["width"] * cfg["height"]
    step = max(1, pixels // npix)
    n = 0
    for pixel in range(0, pixels, step):
        _, work = oracle.pixel_radiance(packed, fs, cfg["width"], cfg["height"], pixel, cfg["seed"] * 7919, topts)
        tot += work
        n += 1
    keys = ["closest_rays", "shadow_rays", "closest_aabb", "closest_tri", "closest_sphere", "closest_nodes",
            "shadow_aabb", "shadow_tri", "shadow_sphere", "shadow_nodes"]
    return {k: float(v) / n for k, v in zip(keys, tot)}


def kernel_bytes_per_step(kernel: str, cpu: dict, units_per_step: int):
    """Algorithmic bytes one step moves through `kernel`, from the reference's work counts.

    Ray queries: 32 B per ray in, 16 B per closest hit out, 32 B per box test,
    48 B per triangle test, 32 B per sphere test (the reference's ordered walk).
    Shading: per closest-hit ray, 16 B hit + 32 B ray in, 48 B primitive +
    64 B material read, 32 B continuation ray out, plus 44 B per shadow ray out.
    Accumulation: 12 B read + 12 B written per sample. Whole paths (k_paths,
    scenes of at most 32 primitives): the ray-query and shading bytes of the
    path together, plus its 16 B radiance written.
    """
    if kernel == "tonemap":  # 12 B of sums read, 4 B of RGBA written per pixel
        return 16 * units_per_step
    if "bytes_per_unit" in cpu:  # traversal workload: one closest-hit query per unit
        return cpu["bytes_per_unit"] * units_per_step if kernel == "closest" else None
    w = cpu["work_per_sample"]
    trace = (w["closest_rays"] * (RAY_BYTES + HIT_BYTES) + w["shadow_rays"] * RAY_BYTES +
             BOX_BYTES * (w["closest_aabb"] + w["shadow_aabb"]) + TRI_BYTES * (w["closest_tri"] + w["shadow_tri"]) +
             SPHERE_BYTES * (w["closest_sphere"] + w["shadow_sphere"]))
    shade = w["closest_rays"] * (16 + 32 + 48 + 64 + 32) + w["shadow_rays"] * 44
    if kernel == "trace":
        per = trace
    elif kernel == "shade":
        per = shade
    elif kernel == "paths":
        per = trace + shade + 16
    elif kernel == "accumulate":
        per = 2 * ACCUM_BYTES_PER_SAMPLE
    else:
        return None
    return per * units_per_step


def workload_name(workload: str, small: bool) -> str:
    if workload == "display":
        c = render_cfg(workload, small)
        return (f"display: tonemapBuffer (ACES, sRGB, RGBA8) of a {c['width']}x{c['height']} sum buffer "
                f"({c['samples']} samples per pixel)")
    if workload == "traversal":
        return ("traversal: 1,000,000-triangle soup, 16,777,216 rays, closest hit" if not small
                else "traversal (small): 100,000 triangles, 1,048,576 rays")
    c = render_cfg(workload, small)
    if workload == "caustic":
        return (f"caustic scene (icosphere level {5 if small else 7} glass blob, 64 spheres, checker ground, "
                f"sphere light) {c['width']}x{c['height']}, {c['spp']} spp, depth {c['max_bounces']}, NEE on, "
                f"RR after bounce 3")
    return f"cornell box {c['width']}x{c['height']}, {c['spp']} spp, depth {c['max_bounces']}, NEE on, RR off"


def workload_config(workload: str, small: bool, gpus: int):
    if workload == "traversal":
        return {"workload": workload_name(workload, small),
                "triangles": 100_000 if small else TRAVERSAL["triangles"],
                "rays": (1 << 20) if small else TRAVERSAL["rays"],
                "l2": "inputs larger than L2 (rays 512 MiB per step)", "parallelism": f"replicas x{gpus}"}
    cfg = render_cfg(workload, small)
    if SIZE_OVERRIDE and workload in ("cornell", "caustic"):
        cfg["size_override"] = True
    return {"workload": workload_name(workload, small), **cfg,
            "l2": "L2 flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{gpus}"}


def reference_record(workload: str, args, steps: int, warmup: int, cpu_seconds: float):
    """The reference algorithm on the host cores for one workload: `warmup`
    untimed and `steps` timed steps, each one bounded sample of the workload
    (sized by a calibration run to cpu_seconds / 4)."""
    import oracle_lib as oracle
    from caustic import _abi

    threads = os.cpu_count() or 1
    rec = cpu_reference(workload, args.small, target_s=cpu_seconds)
    step_s = cpu_seconds / 4
    if workload == "display":
        sums, cfg = display_inputs(args.small)
        w, h = cfg["width"], cfg["height"]
        rows = max(1, min(h, int(rec["value"] * 1e6 * step_s / w)))
        sample = sums[: w * rows * 3]
        units = w * rows

        def step():
            oracle.tonemap(sample, w, rows, cfg["samples"], cfg["exposure_ev"])

        desc = f"{w}x{rows} pixels of the {w}x{h} sum buffer per step, tonemapBuffer (ACES), 1 thread"
        threads = 1
    elif workload == "traversal":
        packed, rays = traversal_inputs(0, args.small, oracle_pack=True)
        n = max(1 << 12, min(len(rays), int(rec["value"] * 1e6 * step_s)))
        sample = rays[:n]
        units = n

        def step():
            oracle.trace(packed, sample, 0, nthreads=threads)

        desc = f"first {n} of the {len(rays)} rays per step, ordered walk (intersectClosest), {threads} threads"
    else:
        packed, frame, cfg = render_inputs(workload, args.small, oracle_pack=True)
        w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
        rows = max(1, min(h, int(rec["value"] * 1e6 * step_s / (w * spp))))
        opts = _abi.ct_render_options(w, rows, spp, cfg["max_bounces"], int(cfg["russian_roulette"]),
                                      int(cfg["nee"]), cfg["seed"])
        fs = frame.struct()
        units = w * rows * spp

        def step():
            oracle.render_image(packed, fs, opts, nthreads=threads)

        desc = f"{w}x{rows} pixels x {spp} spp of the {w}x{h} render per step, {threads} threads"
    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    value = units * steps / dt / 1e6
    metric = {"traversal": "Mrays/s", "display": "Mpixels/s"}.get(workload, "Msamples/s")
    base = {"value": value, "unit": metric, "cores": threads, "kind": "port",
            "sample": desc + "; scenes packed and seeded by the oracle (no CUDA library loaded)"}
    return {
        "impl": "reference", "metric": metric, "value": value, "unit": metric, "n_gpus": args.gpus,
        "steps": steps, "warmup": warmup, "ms_per_step": dt * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(workload, args.small, args.gpus),
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": metric, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference(args, rank, world):
    """The reference arm: the reference algorithm (the oracle, all host threads)
    on rank 0 only. The default line also carries the traversal and caustic
    workloads as sub-records (5 timed steps, 1 warm-up each)."""
    if rank != 0:
        return
    from caustic import _native

    line = reference_record(args.workload, args, args.steps, args.warmup, args.cpu_seconds)
    if default_line(args):
        for sub in SUB_WORKLOADS:
            rec = reference_record(sub, args, min(args.steps, 5), min(args.warmup, 1), args.cpu_seconds)
            line[sub] = {k: rec[k] for k in SUB_KEYS if k in rec}
    try:
        mapped = "libcaustic_gb300" in pathlib.Path("/proc/self/maps").read_text()
    except OSError:
        mapped = None
    line["product_library_loaded"] = bool(_native._lib is not None or mapped)
    print(json.dumps(line), flush=True)


SUB_WORKLOADS = ("traversal", "caustic")
SUB_KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "config", "clocks",
            "gpu_launches", "cpu_baseline", "roofline", "e2e", "stackless")


def default_line(args) -> bool:
    """The default run (the Cornell headline) also measures traversal, caustic,
    batched and served."""
    return args.workload == "cornell" and not args.small and not args.headline_only


BATCH_KEYS = ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config", "clocks", "gpu_launches",
              "plain_sequential", "speedup_vs_plain", "plain_per_frame", "speedup_vs_per_frame", "plain_large_jobs",
              "plain_large_requests", "latency", "e2e")


def run_gpu(args, rank, world):
    import copy

    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    line = measure(args.workload, args, rank, world, args.steps, args.warmup, headline=True)
    if default_line(args):
        # A sub-record that fails is reported as such; the headline line is printed regardless.
        def sub_record(name, fn, keys):
            try:
                rec = fn()
                line[name] = {k: rec[k] for k in keys if k in rec}
            except Exception as exc:  # noqa: BLE001
                line[name] = {"error": f"{type(exc).__name__}: {exc}"[:500]}
                torch.cuda.synchronize()

        for sub in SUB_WORKLOADS:
            sub_record(sub, lambda sub=sub: measure(sub, args, rank, world, args.steps, args.warmup, headline=False),
                       SUB_KEYS)
        # the batched and served forms (BASELINE configs 4 and 5), fewer steps each
        b_args = copy.copy(args)
        b_args.steps, b_args.warmup = max(1, min(args.steps, 5)), min(args.warmup, 3)
        sub_record("batched", lambda: run_batched(b_args, rank, world, emit=False), BATCH_KEYS)
        s_args = copy.copy(b_args)
        s_args.steps, s_args.trace = max(1, min(args.steps, 2)), "c5"
        sub_record("served", lambda: run_served(s_args, rank, world, emit=False), BATCH_KEYS)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure(workload: str, args, rank: int, world: int, steps: int, warmup: int, headline: bool):
    """One workload on this rank's GPU: device-timed steps with inputs
    resident, per-kernel profile, roofline, CPU baseline and e2e."""
    import torch

    import caustic as ct
    from caustic import _native

    device = torch.device("cuda", torch.cuda.current_device())
    lib = _native.lib()
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    hbm_peak, peak_kind = peaks()

    if workload == "traversal":
        packed, rays_np = traversal_inputs(rank, args.small, args.rays)
        n = len(rays_np)
        dev = ct.DeviceScene(packed)
        d_rays = torch.from_numpy(rays_np).to(device)
        d_prim = torch.empty(n, dtype=torch.int32, device=device)
        d_t = torch.empty(n, dtype=torch.float32, device=device)

        def step():
            _native.check(lib.ct_trace_closest_device(dev.handle, _native.ptr(d_rays), n, _native.ptr(d_prim),
                                                      _native.ptr(d_t), None, None, C.c_void_p(stream.cuda_stream)))

        units_per_step, metric = n, "Mrays/s"
    elif workload == "display":
        sums, cfg = display_inputs(args.small)
        w, h = cfg["width"], cfg["height"]
        d_sums = torch.from_numpy(sums).to(device)
        d_rgba = torch.empty(w * h * 4, dtype=torch.uint8, device=device)
        packed, dev = None, None
        mode = {"aces": 0, "reinhard": 1}[cfg["mode"]]

        def step():
            _native.check(lib.ct_tonemap_device(_native.ptr(d_sums), w, h, float(cfg["samples"]),
                                                float(cfg["exposure_ev"]), mode, _native.ptr(d_rgba),
                                                C.c_void_p(stream.cuda_stream)))

        units_per_step, metric = w * h, "Mpixels/s"
    else:
        packed, frame, cfg = render_inputs(workload, args.small)
        dev = ct.DeviceScene(packed)
        w, h = cfg["width"], cfg["height"]
        d_out = torch.empty(w * h * 3, dtype=torch.float32, device=device)
        ropts = ct.RenderOptions(max_bounces=cfg["max_bounces"], russian_roulette=cfg["russian_roulette"],
                                 nee=cfg["nee"], width=w, height=h, spp=cfg["spp"],
                                 seed=cfg["seed"] + 104729 * rank).struct()
        fs = frame.struct()

        def step():
            _native.check(lib.ct_render_image_device(dev.handle, C.byref(fs), C.byref(ropts), _native.ptr(d_out),
                                                     C.c_void_p(stream.cuda_stream)))

        units_per_step, metric = w * h * cfg["spp"], "Msamples/s"

    # warm-up
    with torch.cuda.stream(stream):
        for _ in range(max(3, warmup)):
            step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with ClockSampler(torch.cuda.current_device()) as clocks:
        for k in range(steps):
            if workload != "traversal":
                with torch.cuda.stream(stream):  # L2 flush, ordered before the step's start event
                    flush.fill_(k & 0xFF)
            starts[k].record(stream)
            step()
            ends[k].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = max_over_ranks(sum(step_ms) / 1e3, world, device)
    value = units_per_step * steps * world / total_s / 1e6

    prof = kernel_profile(lib, step, stream, steps)
    wavefront = None
    if headline and workload in ("cornell", "caustic") and packed.prim_count <= 32:
        # the same render through the wavefront kernels (the form every larger scene takes)
        _native.check(lib.ct_scene_set_option(dev.handle, CT_OPT_PATH_KERNEL, 0))
        with torch.cuda.stream(stream):
            for _ in range(3):
                step()
        torch.cuda.synchronize()
        nsteps = max(3, min(steps, 10))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        for k, (w0, w1) in enumerate(ev):
            with torch.cuda.stream(stream):  # L2 flush before the start event, as in the timed steps
                flush.fill_(k & 0xFF)
            w0.record(stream)
            step()
            w1.record(stream)
        torch.cuda.synchronize()
        _native.check(lib.ct_scene_set_option(dev.handle, CT_OPT_PATH_KERNEL, 1))
        wave_s = sum(w0.elapsed_time(w1) for w0, w1 in ev) / 1e3
        wavefront = {"value": units_per_step * nsteps / wave_s / 1e6, "unit": metric,
                     "what": "the same render through the wavefront kernels (generate, trace, shade over "
                             "compacted queues) instead of the whole-path kernel; identical images"}
    stackless = None
    if workload == "traversal":
        # the same rays through the reference's stackless skip-link walk (intersect.ts:290-365)
        prev = lib.ct_set_traversal(1)
        with torch.cuda.stream(stream):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        lib.ct_set_traversal(prev)
        stackless = {"value": units_per_step * 3 / (e0.elapsed_time(e1) / 1e3) / 1e6, "unit": metric,
                     "what": "the same rays through the reference's stackless skip-link walk over its binary "
                             "node array (intersectClosestStackless) instead of the ordered walk over 4-wide "
                             "records; identical hits"}
    launches_per_step = prof.get("launches_per_step") or 0
    clk = clocks.summary()
    line = {
        "metric": metric, "value": value, "unit": metric, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": total_s * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, Rng of the reference)",
        "config": workload_config(workload, args.small, args.gpus), "clocks": clk,
        "gpu_launches": launches_per_step * steps,
    }

    # CPU baseline (rank 0, N = 1): the oracle on a bounded sample; also yields the algorithmic bytes/unit.
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_reference(workload, args.small, target_s=12.0)
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    sm_count = torch.cuda.get_device_properties(device).multi_processor_count
    line["roofline"] = roofline(workload, args.small, prof, cpu, units_per_step, hbm_peak, peak_kind,
                                dev.device_bytes if dev else 0, sm_count, clk.get("sm_mhz"),
                                step_ms=total_s * 1e3 / steps)

    if wavefront:
        line["wavefront"] = wavefront
    if stackless:
        line["stackless"] = stackless
    if not args.no_e2e:
        line["e2e"] = e2e(workload, args, ct, lib, packed, dev, rank, world, device, steps)
    if dev:
        dev.close()
    del flush
    torch.cuda.empty_cache()
    return line


def kernel_profile(lib, step, stream, steps):
    """Per-kernel device times over a few profiled steps (CUDA events around every launch)."""
    import torch

    if not hasattr(lib, "ct_profile_enable"):
        return {}
    lib.ct_profile_enable(1)
    lib.ct_profile_reset()
    nsteps = max(2, min(steps, 5))
    with torch.cuda.stream(stream):
        for _ in range(nsteps):
            step()
    torch.cuda.synchronize()
    names = (C.c_char_p * 32)()
    ms = (C.c_double * 32)()
    counts = (C.c_uint64 * 32)()
    k = lib.ct_profile_read(names, ms, counts, 32)
    lib.ct_profile_enable(0)
    kernels = {names[i].decode(): {"ms": ms[i], "launches": int(counts[i])} for i in range(k)}
    total_launches = sum(v["launches"] for v in kernels.values())
    return {"kernels": kernels, "steps": nsteps, "launches_per_step": total_launches / nsteps}


def compulsory_bytes_per_step(kernel: str, cpu: dict, units_per_step: int):
    """Bytes a trace step must move at least: each ray read (32 B) and each
    closest hit written (16 B); for whole paths (k_paths) each path's 16 B
    radiance written. The scene once per launch is added by the caller."""
    if kernel == "paths":
        return units_per_step * 16
    if kernel == "tonemap":
        return units_per_step * 16
    if kernel not in ("trace", "closest"):
        return None
    if "bytes_per_unit" in cpu:
        return units_per_step * (RAY_BYTES + HIT_BYTES)
    w = cpu["work_per_sample"]
    return units_per_step * (w["closest_rays"] * (RAY_BYTES + HIT_BYTES) + w["shadow_rays"] * RAY_BYTES)


def roofline(workload, small, prof, cpu, units_per_step, peak, peak_kind, scene_bytes, sm_count, sm_mhz,
             step_ms=None):
    """Roofline of the dominant kernel.

    HBM-bound kernels: achieved = the reference algorithm's bytes per launch /
    the kernel's mean CUDA-event duration; beside it the compulsory bytes
    (rays, hits, scene once) and the DRAM bytes ncu measured per launch, each
    also as a fraction of the peak over the same duration.

    The whole-path kernel (k_paths) keeps its scene in L1 and its path state in
    registers, so HBM does not bound it: its roofline is SM instruction issue,
    achieved = warp instructions per launch (ncu) / the mean launch duration
    against one warp instruction per cycle per scheduler (4 per SM) at the
    sampled SM clock. Its HBM figures stay in the `hbm` sub-record.

    Renders of several waves run consecutive waves on several streams, so
    their launches overlap and a launch's CUDA-event window includes time the
    SMs spend on the other waves' kernels. When the kernel's launch windows
    add up to more than the step, achieved is the algorithmic bytes per step
    over the whole step time instead (a lower bound: it charges the other
    kernels' time to this one too); the per-launch figure stays beside it."""
    kernels = prof.get("kernels", {})
    if not kernels:
        return None
    name, k = max(kernels.items(), key=lambda kv: kv[1]["ms"])
    avg_ms = k["ms"] / k["launches"]
    launches_per_step = k["launches"] / prof["steps"]
    per_step = kernel_bytes_per_step(name, cpu, units_per_step) if cpu else None
    algo = per_step / launches_per_step if per_step else None
    comp_step = compulsory_bytes_per_step(name, cpu, units_per_step) if cpu else None
    comp = comp_step / launches_per_step + scene_bytes if comp_step else None
    rec = traffic_record(workload + ("_small" if small else ""))
    rec = rec if rec and rec.get("scope") == name else None
    traffic = rec.get("dram_bytes_per_launch") if rec else None
    achieved = algo / (avg_ms / 1e3) / 1e9 if algo else None
    rate = lambda b: b / (avg_ms / 1e3) / 1e9 / peak if b else None  # noqa: E731
    share = k["ms"] / sum(v["ms"] for v in kernels.values())
    overlapped = bool(step_ms and k["ms"] / prof["steps"] > 1.02 * step_ms)
    per_launch = achieved
    if overlapped and per_step:
        achieved = per_step / (step_ms / 1e3) / 1e9
    hbm = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": (achieved / peak) if achieved else None, "peak_source": f"{peak_kind} hbm_gbs",
           "traffic": traffic, "algorithmic_bytes_per_launch": algo, "avg_launch_ms": avg_ms, "share": share,
           "compulsory_bytes_per_launch": comp, "compulsory_frac": rate(comp), "dram_frac": rate(traffic)}
    if overlapped:
        hbm["achieved_from"] = ("algorithmic bytes per step / step time: the kernel's launches overlap on several "
                                "streams, so their event windows overlap")
        hbm["achieved_per_launch_windows"] = per_launch
        hbm["launch_windows_ms_per_step"] = k["ms"] / prof["steps"]
        hbm["step_ms"] = step_ms
    if name != "paths":
        if rec:
            hbm["traffic_source"] = rec.get("source")
        return hbm
    hbm["note"] = ("14-primitive scene held in L1: the algorithmic bytes are re-read from L1 (frac > 1), and "
                   "dram_frac is the HBM traffic ncu measured per launch")
    clock = float(sm_mhz or 2070.0)
    inst = rec.get("warp_instructions_per_launch") if rec else None
    issue_peak = sm_count * 4 * clock * 1e6 / 1e9
    achieved_issue = inst / (avg_ms / 1e3) / 1e9 if inst else None
    paths_per_launch = units_per_step / launches_per_step
    return {"bound": "issue", "kernel": name, "achieved": achieved_issue, "peak": issue_peak,
            "unit": "G warp instructions/s", "frac": achieved_issue / issue_peak if achieved_issue else None,
            "peak_source": f"{sm_count} SMs x 4 schedulers x 1 warp instruction per cycle at {clock:.0f} MHz "
                           f"(median sampled SM clock)",
            "traffic": traffic, "avg_launch_ms": avg_ms, "share": share,
            "warp_instructions_per_path": inst / paths_per_launch if inst else None,
            "threads_per_warp_instruction": rec.get("threads_per_warp_instruction") if rec else None,
            "instructions_source": rec.get("source") if rec else None, "hbm": hbm}


def e2e(workload, args, ct, lib, packed, dev, rank, world, device, steps):
    """Same metric through the host-pointer C-ABI calls, copies included."""
    import torch

    from caustic import _abi, _native

    steps = max(1, min(steps, 5))
    if workload == "traversal":
        _, rays_np = traversal_inputs(rank, args.small, args.rays)
        n = len(rays_np)
        rays_pin = torch.from_numpy(rays_np).pin_memory()
        prim_pin = torch.empty(n, dtype=torch.int32).pin_memory()
        t_pin = torch.empty(n, dtype=torch.float32).pin_memory()
        stats = _abi.ct_stats()
        parts = {"upload_ms": 0.0, "kernels_ms": 0.0, "wall_ms": 0.0}

        def call():
            t0 = time.perf_counter()
            _native.check(lib.ct_trace_closest(dev.handle, C.c_void_p(rays_pin.data_ptr()), n,
                                               C.c_void_p(prim_pin.data_ptr()), C.c_void_p(t_pin.data_ptr()),
                                               None, None, C.byref(stats)))
            parts["wall_ms"] += (time.perf_counter() - t0) * 1e3
            parts["upload_ms"] += stats.total_ms - stats.kernel_ms
            parts["kernels_ms"] += stats.kernel_ms

        h2d, d2h, units, metric = n * 32, n * 8, n, "Mrays/s"
    elif workload == "display":
        sums, cfg = display_inputs(args.small)
        w, h = cfg["width"], cfg["height"]
        sums_pin = torch.from_numpy(sums).pin_memory()
        rgba_pin = torch.empty(w * h * 4, dtype=torch.uint8).pin_memory()
        d_sums = torch.empty(sums.size, dtype=torch.float32, device=device)
        d_rgba = torch.empty(w * h * 4, dtype=torch.uint8, device=device)
        stream = torch.cuda.current_stream()
        parts = {"wall_ms": 0.0}

        def call():
            t0 = time.perf_counter()
            d_sums.copy_(sums_pin, non_blocking=True)
            _native.check(lib.ct_tonemap_device(_native.ptr(d_sums), w, h, float(cfg["samples"]),
                                                float(cfg["exposure_ev"]), 0, _native.ptr(d_rgba),
                                                C.c_void_p(stream.cuda_stream)))
            rgba_pin.copy_(d_rgba, non_blocking=True)
            stream.synchronize()
            parts["wall_ms"] += (time.perf_counter() - t0) * 1e3

        h2d, d2h, units, metric = sums.nbytes, w * h * 4, w * h, "Mpixels/s"
    else:
        _, frame, cfg = render_inputs(workload, args.small)
        w, h = cfg["width"], cfg["height"]
        out = torch.empty(w * h * 3, dtype=torch.float32).pin_memory()
        ropts = ct.RenderOptions(max_bounces=cfg["max_bounces"], russian_roulette=cfg["russian_roulette"],
                                 nee=cfg["nee"], width=w, height=h, spp=cfg["spp"],
                                 seed=cfg["seed"] + 104729 * rank).struct()
        fs = frame.struct()
        view = packed.view()

        parts = {"scene_create_ms": 0.0, "render_and_copy_ms": 0.0, "scene_destroy_ms": 0.0}

        def call():
            handle = C.c_void_p()
            t0 = time.perf_counter()
            _native.check(lib.ct_scene_create(C.byref(view), C.byref(handle)))
            t1 = time.perf_counter()
            try:
                _native.check(lib.ct_render_image(handle, C.byref(fs), C.byref(ropts),
                                                  C.c_void_p(out.data_ptr()), None))
            finally:
                t2 = time.perf_counter()
                lib.ct_scene_destroy(handle)
                t3 = time.perf_counter()
            parts["scene_create_ms"] += (t1 - t0) * 1e3
            parts["render_and_copy_ms"] += (t2 - t1) * 1e3
            parts["scene_destroy_ms"] += (t3 - t2) * 1e3

        h2d = packed.prims.nbytes + packed.nodes.nbytes + packed.mats.nbytes + packed.lights.nbytes + \
            packed.prim_object.nbytes
        d2h, units, metric = w * h * 12, w * h * cfg["spp"], "Msamples/s"
    call()
    for k in parts:
        parts[k] = 0.0
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        call()
    dt = max_over_ranks(time.perf_counter() - t0, world, device)
    return {"value": units * steps * world / dt / 1e6, "unit": metric, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": steps,
            "breakdown_ms_per_step": {k: v / steps for k, v in parts.items()}}


def batched_inputs(count: int, small: bool):
    """Packed scenes and render sizes of the batched workload (packing runs in parallel threads)."""
    import concurrent.futures as cf

    import caustic as ct

    spec = ct.batch_workload(count, max_tris=20_000 if small else 200_000)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        packed = list(ex.map(lambda s: ct.pack_scene(s[0]), spec))
    return [(p, ct.camera_frame(s.camera, w / h), w, h) for p, (s, w, h) in zip(packed, spec)]


def run_batched(args, rank, world, emit=True):
    """Batched form: all jobs in one graph launch vs the same jobs as sequential plain renders."""
    import torch

    import caustic as ct
    from caustic import _native

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    device = torch.device("cuda", torch.cuda.current_device())
    spp = 4 if args.small else 16
    opts = ct.TraceOptions(max_bounces=8, russian_roulette=True, nee=True)
    inputs = batched_inputs(args.jobs, args.small)
    scenes = [ct.DeviceScene(p) for p, _, _, _ in inputs]
    jobs = [ct.Job(d, f, w, h, spp, seed=1 + i + 1000 * rank) for i, (d, (_, f, w, h)) in enumerate(zip(scenes, inputs))]
    samples = sum(j.width * j.height * spp for j in jobs)
    stream = torch.cuda.Stream()
    br = ct.BatchRenderer(jobs, opts)
    lib = _native.lib()
    outs = [torch.empty(j.width * j.height * 3, device=device) for j in jobs]
    ropts = [ct.RenderOptions(max_bounces=8, russian_roulette=True, nee=True, width=j.width, height=j.height,
                              spp=spp, seed=j.seed).struct() for j in jobs]
    fstructs = [j.frame.struct() for j in jobs]

    def batched_step():
        br.run(stream)

    def plain_step():
        for j, o, f, out in zip(jobs, ropts, fstructs, outs):
            _native.check(lib.ct_render_image_device(j.scene.handle, C.byref(f), C.byref(o), _native.ptr(out),
                                                     C.c_void_p(stream.cuda_stream)))

    topts = opts.struct()
    spp_div = torch.full((), float(spp), dtype=torch.float32, device=device)  # true division, as renderImage

    def per_frame_step():
        # each job as a progressive loop: one accumulatePass per frame, then / spp
        with torch.cuda.stream(stream):
            for j, f, out in zip(jobs, fstructs, outs):
                out.zero_()
                for k in range(spp):
                    _native.check(lib.ct_accumulate_passes_device(
                        j.scene.handle, C.byref(f), j.width, j.height, (j.seed * 7919 + k) & 0xFFFFFFFF, 1,
                        C.byref(topts), _native.ptr(out), None, C.c_void_p(stream.cuda_stream)))
                out.div_(spp_div)

    def timed(step, steps):
        with torch.cuda.stream(stream):
            for _ in range(max(3, args.warmup)):
                step()
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / 1e3, world, device)

    with ClockSampler(torch.cuda.current_device()) as clocks:
        t_batch = timed(batched_step, args.steps)
    t_plain = timed(plain_step, max(1, args.steps // 2))
    plain_rate = samples * max(1, args.steps // 2) * world / t_plain / 1e6
    # The plain loop on the jobs of at least FILL_PATHS paths alone: they
    # fill the GPU by themselves and hold most of the samples, so the gap
    # between this rate and the batched rate is what batching gains on them
    # (bounce tails and per-render launches), not on small jobs.
    big = [k for k, j in enumerate(jobs) if j.width * j.height * spp >= FILL_PATHS]

    def plain_big_step():
        for k in big:
            j = jobs[k]
            _native.check(lib.ct_render_image_device(j.scene.handle, C.byref(fstructs[k]), C.byref(ropts[k]),
                                                     _native.ptr(outs[k]), C.c_void_p(stream.cuda_stream)))

    t_big = timed(plain_big_step, max(1, args.steps // 2)) if big else 0.0
    t_frame = timed(per_frame_step, 1)
    frame_rate = samples * world / t_frame / 1e6
    value = samples * args.steps * world / t_batch / 1e6
    # end to end: graph launch + copy of every job's sums into pinned host
    # buffers (asynchronous on the render stream, one wait per step)
    host = [torch.empty(a.shape, dtype=a.dtype, pin_memory=True) for a in br.accums]
    t0 = time.perf_counter()
    for _ in range(2):
        br.run(stream)
        with torch.cuda.stream(stream):
            for h, a in zip(host, br.accums):
                h.copy_(a, non_blocking=True)
        stream.synchronize()
    e2e_rate = samples * 2 * world / (time.perf_counter() - t0) / 1e6
    info = br.info()
    line = {
        "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_batch * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, Rng of the reference)",
        "config": {"workload": f"batched: {len(jobs)} scenes (soups of 2k-{20_000 if args.small else 200_000} "
                               f"triangles, 0-32 spheres, quad light), sizes 64-512 squared, {spp} spp, depth 8, "
                               f"one CUDA graph per run",
                   "jobs": len(jobs), "triangles": int(sum(p.prim_count for p, _, _, _ in inputs)),
                   "samples_per_step": samples, "waves": info["waves"], "graph_nodes": info["graph_nodes"],
                   "walk": info["walk"], "parallelism": f"replicas x{args.gpus}"},
        "plain_sequential": {"value": plain_rate, "unit": "Msamples/s",
                             "what": "the same jobs as consecutive ct_render_image_device calls"},
        "speedup_vs_plain": value / plain_rate,
        "plain_large_jobs": {
            "value": (sum(jobs[k].width * jobs[k].height * spp for k in big) * max(1, args.steps // 2) * world
                      / t_big / 1e6) if t_big else None, "unit": "Msamples/s", "jobs": len(big),
            "share_of_samples": sum(jobs[k].width * jobs[k].height * spp for k in big) / samples,
            "share_of_plain_time": t_big / t_plain if t_big else None,
            "what": f"the plain loop on the jobs of at least {FILL_PATHS} paths alone (they fill the GPU by "
                    "themselves)"},
        "plain_per_frame": {"value": frame_rate, "unit": "Msamples/s",
                            "what": "the same jobs one after another, each as a progressive loop of one "
                                    "accumulatePass per frame (ct_accumulate_passes_device, passes = 1)"},
        "speedup_vs_per_frame": value / frame_rate,
        "clocks": clocks.summary(),
        # kernel nodes of the graph (all nodes but one counter memset per wave), one replay per step
        "gpu_launches": (info["graph_nodes"] - info["waves"]) * args.steps,
        "e2e": {"value": e2e_rate, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(sum(j.width * j.height * 12 for j in jobs)),
                "what": "graph launch + device-to-host copy of all sums into pinned host buffers; scenes stay "
                        "resident"},
    }
    br.close()
    for d in scenes:
        d.close()
    if emit and rank == 0:
        print(json.dumps(line), flush=True)
    return line


def served_inputs(count: int, small: bool, rank: int, trace: str = "c5"):
    """Scene pool and request trace of the served workload. Pool: the 256
    batched-workload soups, the unit Cornell box and the caustic scene.
    Requests: `count`, each drawing a scene from the pool, a square side in
    128..1024 (multiples of 128) and a target spp log-uniform in [1, 256]
    (Rng(4242 + rank)); arrivals Poisson of mean gap 1 (rescaled by the caller)."""
    import concurrent.futures as cf

    import caustic as ct
    from caustic.serve import poisson_requests

    soups = ct.batch_workload(32 if small else 256, max_tris=20_000 if small else 200_000)
    pool = {"cornell": ct.cornell_unit_box(), "caustic": ct.caustic_scene(level=5 if small else 7)}
    pool.update({f"soup{i}": s for i, (s, _, _) in enumerate(soups)})
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        packed = dict(zip(pool, ex.map(ct.pack_scene, pool.values())))
    frames = {k: (lambda a, cam=s.camera: ct.camera_frame(cam, a)) for k, s in pool.items()}
    if trace == "preview":  # interactive previews: small images, few passes
        sides, max_spp = (128, 192, 256), 8
    else:
        sides, max_spp = ((128, 256, 384), 64) if small else (tuple(range(128, 1025, 128)), 256)
    reqs = poisson_requests(list(pool), frames, count, rate=1.0, seed=4242 + rank, sides=sides, max_spp=max_spp)
    return packed, reqs


def run_served(args, rank, world, emit=True):
    """Served form: a request trace through the continuous-batching server
    against the same trace as one plain renderImage per request, first all
    queued at once (throughput), then with Poisson arrivals (latency)."""
    import copy

    import torch

    import caustic as ct
    from caustic.serve import GpuExecutor, RenderServer, latency_stats, render_per_frame, render_plain

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    device = torch.device("cuda", torch.cuda.current_device())
    opts = ct.TraceOptions(max_bounces=8, russian_roulette=True, nee=True)
    count = 32 if args.small else args.requests
    packed, trace = served_inputs(count, args.small, rank, args.trace)
    dev = {k: ct.DeviceScene(p) for k, p in packed.items()}
    samples = sum(r.pixels * r.spp for r in trace)

    def at(reqs, rate):
        # the trace's arrival pattern scaled to `rate` requests/s (rate=None: all at t=0)
        out = copy.deepcopy(reqs)
        for r in out:
            r.arrival = 0.0 if rate is None else r.arrival / rate
        return out

    def served(rate=None, policy="round_robin"):
        ex = GpuExecutor(dev, opts)
        srv = RenderServer(ex, policy=policy)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(ex.stream)
        res = srv.serve(at(trace, rate), t0=t0)
        e1.record(ex.stream)
        torch.cuda.synchronize()
        return res, time.perf_counter() - t0, e0.elapsed_time(e1) / 1e3, srv

    def plain(rate=None):
        t0 = time.perf_counter()
        res = render_plain(dev, at(trace, rate), opts, t0=t0)
        torch.cuda.synchronize()
        return res, time.perf_counter() - t0

    def per_frame(rate=None):
        t0 = time.perf_counter()
        res = render_per_frame(dev, at(trace, rate), opts, t0=t0)
        torch.cuda.synchronize()
        return res, time.perf_counter() - t0

    for _ in range(max(3, args.warmup)):
        served()
    plain()
    torch.cuda.synchronize()
    barrier(world)
    walls, devs = [], []
    with ClockSampler(torch.cuda.current_device()) as clocks:
        for _ in range(args.steps):
            res, wall, dev_t, srv = served()
            walls.append(wall)
            devs.append(dev_t)
    t_dev = max_over_ranks(sum(devs), world, device)
    t_wall = max_over_ranks(sum(walls), world, device)
    _, t_plain = plain()
    t_plain = max_over_ranks(t_plain, world, device)
    value = samples * args.steps * world / t_dev / 1e6
    plain_rate = samples * world / t_plain / 1e6
    # The plain loop on the requests of at least FILL_PATHS paths alone (as in
    # the batched workload).
    big = [r for r in trace if r.pixels * r.spp >= FILL_PATHS]
    t0 = time.perf_counter()
    render_plain(dev, at(big, None), opts, t0=t0)
    torch.cuda.synchronize()
    t_big = max_over_ranks(time.perf_counter() - t0, world, device) if big else 0.0
    _, t_frame = per_frame()
    t_frame = max_over_ranks(t_frame, world, device)
    frame_rate = samples * world / t_frame / 1e6
    # latency under Poisson arrivals at 80% of the plain path's request capacity
    rate = 0.8 * len(trace) / t_plain
    res_s, _, _, srv_s = served(rate)
    res_f, _, _, _ = served(rate, "fifo")
    res_r, _, _, _ = served(rate, "srpt")
    res_a, _, _, _ = served(rate, "srpt_age")
    res_p, _ = plain(rate)
    if args.trace == "preview":
        mix = "preview mix: sides 128-256 squared, 1-8 spp"
    else:
        mix = (f"sides {'128-384' if args.small else '128-1024'} squared, 1-{64 if args.small else 256} spp")
    line = {
        "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, Rng of the reference)",
        "config": {"workload": f"served: {len(trace)} requests over {len(dev)} resident scenes (batched-workload "
                               f"soups, unit Cornell box, caustic scene), {mix}, depth 8, continuous batching of "
                               f"progressive passes (16 Mi paths per step, four steps in flight on four streams, round robin), all "
                               f"requests queued at t=0",
                   "requests": len(trace), "scenes": len(dev), "samples_per_step": samples,
                   "server_steps": srv.steps, "peak_device_bytes": srv.peak_bytes,
                   "parallelism": f"replicas x{args.gpus}"},
        "plain_sequential": {"value": plain_rate, "unit": "Msamples/s",
                             "what": "the same requests as consecutive ct_render_image_device calls, one at a time"},
        "speedup_vs_plain": value / plain_rate,
        "plain_large_requests": {
            "value": sum(r.pixels * r.spp for r in big) * world / t_big / 1e6 if t_big else None,
            "unit": "Msamples/s", "requests": len(big),
            "share_of_samples": sum(r.pixels * r.spp for r in big) / samples,
            "share_of_plain_time": t_big / t_plain if t_big else None,
            "what": f"the plain loop on the requests of at least {FILL_PATHS} paths alone (they fill the GPU by "
                    "themselves)"},
        "plain_per_frame": {"value": frame_rate, "unit": "Msamples/s",
                            "what": "the same requests one at a time, each as a progressive loop of one "
                                    "accumulatePass per frame (ct_accumulate_passes_device, passes = 1)"},
        "speedup_vs_per_frame": value / frame_rate,
        "latency": {"arrivals": f"Poisson, {rate:.1f} requests/s (80% of the plain path's capacity)",
                    "served": latency_stats(res_s), "served_fifo": latency_stats(res_f),
                    "served_srpt": latency_stats(res_r), "served_srpt_age": latency_stats(res_a),
                    "plain": latency_stats(res_p),
                    "served_steps": srv_s.steps},
        "clocks": clocks.summary(),
        "e2e": {"value": samples * args.steps * world / t_wall / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(sum(r.buffer_bytes for r in trace)),
                "what": "host clock around the whole serve loop: batch planning, launches, per-step synchronisation "
                        "and the device-to-host read of every finished image; scenes stay resident"},
    }
    for d in dev.values():
        d.close()
    if emit and rank == 0:
        print(json.dumps(line), flush=True)
    return line


def main():
    global SIZE_OVERRIDE
    args = parse_args()
    if args.size:
        SIZE_OVERRIDE = tuple(int(x) for x in args.size.lower().split("x"))
    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if args.impl == "gb300" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        elif args.workload == "batched":
            run_batched(args, rank, world)
        elif args.workload == "served":
            run_served(args, rank, world)
        else:
            run_gpu(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Render serving with continuous batching.

Requests (scene, camera, size, target spp, seed) arrive over time. The
server keeps scenes (BVHs) and each admitted request's accumulation buffer
resident on the device and, every step, advances admitted requests by a
progressive chunk of passes in one batched launch (ct_batch_run_direct).
A request is admitted, in arrival order, as soon as its buffer fits in the
device-memory budget next to the resident scenes, the other admitted
requests and the path state of the steps in flight; it leaves when its last
pass has completed, freeing its memory for waiting requests. Steps are
pipelined two deep: the host plans and launches step k+1 while step k runs,
then completes step k. Request r's pass k always uses frame index
seed*7919 + k (tracer.ts:351), so its image does not depend on which other
requests shared its steps.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass
from typing import Callable, Deque, Dict, Iterable, List, Optional, Protocol, Sequence

import numpy as np

from .camera import CameraFrame
from .tracer import DeviceScene, TraceOptions

PATH_STATE_BYTES = 200  # device bytes per path slot in flight (queues, radiance, hit, job ids)
# Steps in flight (each on its own stream) and paths per step: on the C5
# trace, 8 Mi paths two deep 1,011 Msamples/s, three deep 1,066; 16 Mi paths
# two deep 1,075, three 1,112, four 1,159; 24 Mi three deep 1,133.
STEPS_IN_FLIGHT = 4


@dataclass
class Request:
    rid: int
    scene: str
    frame: CameraFrame
    width: int
    height: int
    spp: int
    seed: int = 0
    arrival: float = 0.0  # seconds on the server clock

    @property
    def pixels(self) -> int:
        return self.width * self.height

    @property
    def buffer_bytes(self) -> int:
        return self.pixels * 12


@dataclass
class Result:
    request: Request
    image: Optional[np.ndarray]  # None unless status == "done"
    admitted: Optional[float]    # None for a request cancelled before admission
    finished: float
    status: str = "done"         # "done", "cancelled" or "failed"
    error: Optional[str] = None

    @property
    def latency(self) -> float:
        return self.finished - self.request.arrival


@dataclass
class _Active:
    req: Request
    seq: int = 0     # admission order
    issued: int = 0  # passes launched
    done: int = 0    # passes completed
    admitted: float = 0.0
    buffer: object = None
    inflight: int = 0                # steps in flight that hold passes of this request
    stop: Optional[str] = None       # "cancelled" or "failed": leaves once nothing is in flight
    error: Optional[str] = None


class Executor(Protocol):
    """Device side of the server (a fake one drives the scheduler in tests)."""

    def scene_bytes(self, name: str) -> int: ...
    def walk_class(self, name: str) -> int: ...   # requests of one class share a step
    def allocate(self, req: Request): ...
    def launch(self, items: Sequence[tuple]): ...   # (request, buffer, first pass, passes) -> ticket
    def wait(self, ticket) -> None: ...
    def fetch(self, req: Request, buffer) -> Optional[np.ndarray]: ...
    def release(self, buffer) -> None: ...


class RenderServer:
    POLICIES = ("round_robin", "fifo", "srpt", "srpt_age")

    def __init__(self, executor: Executor, budget_bytes: int = 120 << 30, step_paths: int = 16 << 20,
                 min_chunk_paths: int = 16 << 20, max_passes_per_step: Optional[int] = None,
                 clock: Callable[[], float] = time.perf_counter, policy: str = "round_robin",
                 age_limit: float = 0.10):
        if policy not in self.POLICIES:
            raise ValueError(f"policy {policy!r} is not one of {self.POLICIES}")
        self.policy = policy
        self.age_limit = float(age_limit)
        self.ex = executor
        self.budget = int(budget_bytes)
        self.step_paths = int(step_paths)
        self.min_chunk = int(min_chunk_paths)
        self.max_passes = max_passes_per_step
        self.clock = clock
        self.waiting: Deque[Request] = deque()
        self.active: List[_Active] = []
        self.inflight: Deque[tuple] = deque()  # (ticket, [(active, passes)])
        self.results: List[Result] = []
        self.scenes_in_use: Dict[str, int] = {}
        self.peak_bytes = 0
        self.steps = 0
        self.samples = 0
        self._seq = 0
        self._next = 0  # admission number the next step starts from (round robin)

    # -- admission -----------------------------------------------------------
    def _path_bytes(self) -> int:
        return STEPS_IN_FLIGHT * self.step_paths * PATH_STATE_BYTES

    def resident_bytes(self) -> int:
        scenes = sum(self.ex.scene_bytes(s) for s in self.scenes_in_use)
        return scenes + sum(a.req.buffer_bytes for a in self.active) + self._path_bytes()

    def submit(self, req: Request) -> None:
        self.waiting.append(req)

    def cancel(self, rid: int) -> bool:
        """Cancels request `rid`: a waiting request leaves at once; an admitted
        one takes no further passes and leaves (its buffer released) when the
        steps in flight that hold its passes have completed. Returns whether
        the request was found."""
        for req in list(self.waiting):
            if req.rid == rid:
                self.waiting.remove(req)
                self.results.append(Result(req, None, None, self.clock(), "cancelled"))
                return True
        for a in self.active:
            if a.req.rid == rid and a.stop is None:
                a.stop = "cancelled"
                if a.inflight == 0:
                    self._retire(a)
                return True
        return False

    def _retire(self, a: _Active, image=None) -> None:
        status = a.stop or "done"
        self.results.append(Result(a.req, image if status == "done" else None, a.admitted, self.clock(), status,
                                   a.error))
        self.ex.release(a.buffer)
        self.active.remove(a)
        n = self.scenes_in_use[a.req.scene] - 1
        if n:
            self.scenes_in_use[a.req.scene] = n
        else:
            del self.scenes_in_use[a.req.scene]

    def _fail(self, plan, err: Exception) -> None:
        for a, _ in plan:
            if a.stop is None:
                a.stop, a.error = "failed", f"{type(err).__name__}: {err}"
            if a.inflight == 0 and a in self.active:
                self._retire(a)

    def _admit(self) -> None:
        while self.waiting:
            req = self.waiting[0]
            if req.buffer_bytes + self.ex.scene_bytes(req.scene) + self._path_bytes() > self.budget:
                raise ValueError(f"request {req.rid} alone exceeds the device-memory budget")
            extra = req.buffer_bytes + (0 if req.scene in self.scenes_in_use else self.ex.scene_bytes(req.scene))
            if self.active and self.resident_bytes() + extra > self.budget:
                break  # wait for memory; an idle server always admits the head request
            self.waiting.popleft()
            self.scenes_in_use[req.scene] = self.scenes_in_use.get(req.scene, 0) + 1
            self.active.append(_Active(req, self._seq, 0, 0, self.clock(), self.ex.allocate(req)))
            self._seq += 1
            self.peak_bytes = max(self.peak_bytes, self.resident_bytes())

    # -- scheduling ------------------------------------------------------------
    def _plan(self) -> list:
        """One step: requests with passes left, all of the first one's walk
        class, packed into at most step_paths paths (one wave). Order: round
        robin from where the last step stopped (small requests finish within a
        few steps of arriving; large ones share the GPU), fifo: always from
        the oldest (a large request runs as fast as alone, later ones only fill
        what is left of each wave), or srpt: the fewest samples left first
        (small requests go ahead of large ones, and a large request is not
        spread over the steps of many others; ties by admission order), or
        srpt_age: srpt among the requests that arrived less than age_limit
        seconds ago, every older one first in admission order (a large
        request waits at most about age_limit behind smaller ones). Each request gets an equal share of the
        step, but at least min_chunk_paths (a request's chunk keeps its scene
        hot in L2 for a while) and at least one pass, at most what it still
        needs and what still fits; requests that do not fit wait for the next
        step, which under round robin starts at the first of them."""
        pending = [a for a in self.active if a.issued < a.req.spp and a.stop is None]
        if not pending:
            return []
        pending.sort(key=lambda a: a.seq)
        if self.policy == "round_robin":
            k = next((i for i, a in enumerate(pending) if a.seq >= self._next), 0)
            pending = pending[k:] + pending[:k]
        elif self.policy == "srpt":
            pending.sort(key=lambda a: ((a.req.spp - a.issued) * a.req.pixels, a.seq))
        elif self.policy == "srpt_age":
            now = self.clock()
            pending.sort(key=lambda a: (0, a.seq, 0) if now - a.req.arrival > self.age_limit
                         else (1, (a.req.spp - a.issued) * a.req.pixels, a.seq))
        cls = self.ex.walk_class(pending[0].req.scene)
        share = max(self.step_paths / len(pending), min(self.min_chunk, self.step_paths))
        room = self.step_paths
        plan, skipped = [], None
        for a in pending:
            if self.ex.walk_class(a.req.scene) != cls:
                skipped = a if skipped is None else skipped
                continue
            px = max(1, a.req.pixels)
            want = max(1, min(a.req.spp - a.issued, int(share // px)))
            if self.max_passes:
                want = min(want, self.max_passes)
            fit = room // px
            if fit == 0 and plan:
                skipped = a if skipped is None else skipped
                continue
            p = max(1, min(want, fit))  # a pass larger than a whole step goes alone (split by pixels)
            plan.append((a, p))
            room -= p * px
            if room <= 0:
                break
        last = plan[-1][0]
        after = [a for a in pending if a.seq > last.seq]
        self._next = skipped.seq if skipped is not None else (after[0].seq if after else 0)
        return plan

    def _complete_oldest(self) -> int:
        ticket, plan = self.inflight.popleft()
        for a, _ in plan:
            a.inflight -= 1
        try:
            self.ex.wait(ticket)
        except Exception as err:  # the step failed on the device: its requests fail, the server goes on
            self._fail(plan, err)
            return 0
        rendered = 0
        for a, p in plan:
            if a not in self.active:
                continue
            a.done += p
            rendered += p * a.req.pixels
            if a.stop is not None:
                if a.inflight == 0:
                    self._retire(a)
            elif a.done >= a.req.spp:
                self._retire(a, self.ex.fetch(a.req, a.buffer))
        self.samples += rendered
        return rendered

    def step(self) -> int:
        """Admits what fits, launches the next step, completes the oldest step
        in flight once STEPS_IN_FLIGHT are queued (or nothing is left to
        launch). Returns the samples completed."""
        self._admit()
        plan = self._plan()
        if plan:
            try:
                ticket = self.ex.launch([(a.req, a.buffer, a.issued, p) for a, p in plan])
            except Exception as err:  # e.g. a failed upload or launch: these requests fail
                self._fail(plan, err)
                plan = []
            else:
                for a, p in plan:
                    a.issued += p
                    a.inflight += 1
                self.inflight.append((ticket, plan))
                self.steps += 1
        if self.inflight and (len(self.inflight) >= STEPS_IN_FLIGHT or not plan):
            return self._complete_oldest()
        return 0

    def __len__(self) -> int:
        return len(self.waiting) + len(self.active)

    def busy(self) -> bool:
        return bool(self.waiting or self.active or self.inflight)

    def drain(self) -> List[Result]:
        while self.busy():
            self.step()
        return self.results

    def serve(self, requests: Iterable[Request], t0: Optional[float] = None) -> List[Result]:
        """Replays `requests` (arrival times relative to t0) in real time until all finish."""
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = self.clock() if t0 is None else t0
        for r in pending:
            r.arrival += t0
        i = 0
        while i < len(pending) or self.busy():
            now = self.clock()
            while i < len(pending) and pending[i].arrival <= now:
                self.submit(pending[i])
                i += 1
            if not self.busy():
                time.sleep(max(0.0, min(0.01, pending[i].arrival - now)))
                continue
            self.step()
        return self.results


def latency_stats(results: Sequence[Result]) -> dict:
    """Latency percentiles (ms) of the completed requests."""
    lat = np.array([r.latency for r in results if r.status == "done"], dtype=np.float64) * 1e3
    if len(lat) == 0:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max())}


class GpuExecutor:
    """Executor on libcaustic_gb300: device-resident scenes and sum buffers, one
    ct_batch per step launched without graph capture. Consecutive steps run on
    `streams` streams in turn, so a step's last bounces overlap the next
    step's first ones; each step's sums are added after the previous step's
    (ct_batch_run_direct_after), which keeps every request's passes in pass
    order. Finished images are read back on a copy stream while the next step
    runs."""

    def __init__(self, scenes: Dict[str, DeviceScene], opts: TraceOptions, wave_paths: int = 0, stream=None,
                 streams: int = STEPS_IN_FLIGHT):
        import torch

        from . import _abi, _native

        self.scenes = scenes
        self.opts = opts
        self.wave_paths = wave_paths
        self._lib = _native.lib()
        self._abi = _abi
        self._native = _native
        self.stream = stream or torch.cuda.Stream()  # sum buffers are zeroed here; steps 0, n, 2n, ... run here
        self.streams = [self.stream] + [torch.cuda.Stream() for _ in range(max(1, streams) - 1)]
        self._turn = 0
        self._last = None  # the previous step's batch (alive until the server waits for it)
        self.copy_stream = torch.cuda.Stream()
        self._topts = _abi.ct_trace_options(opts.max_bounces, int(opts.russian_roulette), int(opts.nee))
        self._bytes = {k: v.device_bytes for k, v in scenes.items()}
        self._walk = {k: v.walk for k, v in scenes.items()}

    def scene_bytes(self, name: str) -> int:
        return self._bytes[name]

    def walk_class(self, name: str) -> int:
        # ct_batch gives each trace walk waves of its own: a step of one walk is one wave
        return self._walk[name]

    def allocate(self, req: Request):
        import torch

        with torch.cuda.stream(self.stream):  # zeroed in order with the steps that add to it
            return torch.zeros(req.pixels * 3, dtype=torch.float32, device="cuda")

    def launch(self, items):
        import ctypes as C

        arr = (self._abi.ct_batch_job * len(items))()
        for k, (req, buf, first, passes) in enumerate(items):
            arr[k].scene = self.scenes[req.scene].handle
            arr[k].frame = req.frame.struct()
            arr[k].width, arr[k].height = req.width, req.height
            arr[k].first_frame_index = (req.seed * 7919 + first) & 0xFFFFFFFF
            arr[k].passes = passes
            arr[k].accum = buf.data_ptr()
        handle = C.c_void_p()
        self._native.check(self._lib.ct_batch_create(arr, len(items), C.byref(self._topts), self.wave_paths, -1,
                                                     C.byref(handle)))
        s = self.streams[self._turn % len(self.streams)]
        if s is not self.stream:  # the sum buffers zeroed so far, before this step adds to them
            s.wait_stream(self.stream)
        try:
            self._native.check(self._lib.ct_batch_run_direct_after(handle, C.c_void_p(s.cuda_stream), self._last))
        except Exception:
            self._lib.ct_batch_destroy(handle)
            raise
        self._turn += 1
        self._last = handle
        return handle

    def wait(self, handle) -> None:
        if self._last is not None and self._last.value == handle.value:
            self._last = None
        self._lib.ct_batch_destroy(handle)  # waits for the batch's run, recycles its buffers

    def fetch(self, req: Request, buf) -> np.ndarray:
        import torch

        from .batch import divide_exact

        with torch.cuda.stream(self.copy_stream):
            out = divide_exact(buf, req.spp).cpu()
        return out.numpy()

    def release(self, buf) -> None:
        del buf


def render_plain(scenes: Dict[str, DeviceScene], requests: Sequence[Request], opts: TraceOptions,
                 clock: Callable[[], float] = time.perf_counter, t0: Optional[float] = None) -> List[Result]:
    """The per-request baseline: requests served one at a time in arrival order,
    each a full renderImage (ct_render_image_device), no batching."""
    import ctypes as C

    import torch

    from . import _native
    from .tracer import RenderOptions

    lib = _native.lib()
    stream = torch.cuda.Stream()
    t0 = clock() if t0 is None else t0
    results = []
    for req in sorted(requests, key=lambda r: r.arrival):
        arrival = t0 + req.arrival
        while clock() < arrival:
            time.sleep(max(0.0, min(0.01, arrival - clock())))
        start = clock()
        out = torch.empty(req.pixels * 3, dtype=torch.float32, device="cuda")
        o = RenderOptions(max_bounces=opts.max_bounces, russian_roulette=opts.russian_roulette, nee=opts.nee,
                          width=req.width, height=req.height, spp=req.spp, seed=req.seed).struct()
        f = req.frame.struct()
        _native.check(lib.ct_render_image_device(scenes[req.scene].handle, C.byref(f), C.byref(o), _native.ptr(out),
                                                 C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        img = out.cpu().numpy()
        r = Request(req.rid, req.scene, req.frame, req.width, req.height, req.spp, req.seed, arrival)
        results.append(Result(r, img, start, clock()))
    return results


def render_per_frame(scenes: Dict[str, DeviceScene], requests: Sequence[Request], opts: TraceOptions,
                     clock: Callable[[], float] = time.perf_counter, t0: Optional[float] = None) -> List[Result]:
    """The per-frame baseline: requests served one at a time in arrival order,
    each as the reference's progressive loop renders it, one accumulatePass
    (ct_accumulate_passes_device with passes = 1) per frame with frame index
    seed*7919 + k (tracer.ts:351), then divided by spp. The frames are
    queued back to back on one stream; the host waits once per request."""
    import ctypes as C

    import torch

    from . import _native
    from .batch import divide_exact

    lib = _native.lib()
    stream = torch.cuda.Stream()
    t0 = clock() if t0 is None else t0
    o = opts.struct()
    results = []
    for req in sorted(requests, key=lambda r: r.arrival):
        arrival = t0 + req.arrival
        while clock() < arrival:
            time.sleep(max(0.0, min(0.01, arrival - clock())))
        start = clock()
        f = req.frame.struct()
        with torch.cuda.stream(stream):
            accum = torch.zeros(req.pixels * 3, dtype=torch.float32, device="cuda")
            for k in range(req.spp):
                _native.check(lib.ct_accumulate_passes_device(
                    scenes[req.scene].handle, C.byref(f), req.width, req.height,
                    (req.seed * 7919 + k) & 0xFFFFFFFF, 1, C.byref(o), _native.ptr(accum), None,
                    C.c_void_p(stream.cuda_stream)))
            accum = divide_exact(accum, req.spp)
        stream.synchronize()
        img = accum.cpu().numpy()
        r = Request(req.rid, req.scene, req.frame, req.width, req.height, req.spp, req.seed, arrival)
        results.append(Result(r, img, start, clock()))
    return results


def poisson_requests(names: Sequence[str], frames: Dict[str, Callable[[float], CameraFrame]], count: int,
                     rate: float, seed: int = 99, sides=(128, 256, 384, 512, 768, 1024), max_spp: int = 256):
    """`count` requests with exponential inter-arrival times of mean 1/rate: a
    scene drawn uniformly from `names`, a square side from `sides`, a target
    spp log-uniform in [1, max_spp] (all draws from the reference's Rng)."""
    from .rng import Rng

    rng = Rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += -math.log(1.0 - rng.next()) / rate
        name = names[rng.int(len(names))]
        side = sides[rng.int(len(sides))]
        spp = max(1, int(round(math.exp(rng.range(0.0, math.log(max_spp))))))
        out.append(Request(i, name, frames[name](1.0), side, side, spp, seed=1 + i, arrival=t))
    return out

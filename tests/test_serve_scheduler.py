"""Serving scheduler (host logic) with a fake executor: admission by memory
budget, progressive chunks, retirement, and the waiting queue."""
import pytest

import caustic as ct
from caustic.serve import PATH_STATE_BYTES, STEPS_IN_FLIGHT, RenderServer, Request


class FakeExecutor:
    def __init__(self, scene_bytes):
        self.sb = scene_bytes
        self.steps = []
        self.live = set()
        self.peak_live = 0

    def scene_bytes(self, name):
        return self.sb[name]

    def walk_class(self, name):
        return 1 if name.startswith("skip") else 0

    def allocate(self, req):
        self.live.add(req.rid)
        self.peak_live = max(self.peak_live, len(self.live))
        return {"rid": req.rid, "passes": []}

    def launch(self, items):
        self.steps.append([(r.rid, first, p) for r, _, first, p in items])
        self.pending = getattr(self, "pending", 0) + 1
        for r, buf, first, p in items:
            buf["passes"].append((first, p))
        return len(self.steps)

    def wait(self, ticket):
        self.pending -= 1
        self.waited = getattr(self, "waited", []) + [ticket]

    def fetch(self, req, buf):
        return buf["passes"]

    def release(self, buf):
        self.live.discard(buf["rid"])


def _req(rid, side, spp, scene="a", arrival=0.0):
    frame = ct.camera_frame(ct.CORNELL_BOX.camera, 1.0)
    return Request(rid, scene, frame, side, side, spp, seed=rid, arrival=arrival)


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def test_every_request_gets_exactly_its_passes_in_order():
    ex = FakeExecutor({"a": 1000, "b": 2000})
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=64 * 64 * 4, clock=Clock())
    reqs = [_req(0, 64, 10), _req(1, 32, 3, "b"), _req(2, 128, 7), _req(3, 16, 1)]
    for r in reqs:
        srv.submit(r)
    srv.drain()
    assert sorted(r.request.rid for r in srv.results) == [0, 1, 2, 3]
    assert ex.waited == sorted(ex.waited) and ex.pending == 0  # steps complete in launch order
    for res in srv.results:
        passes = res.image
        # contiguous progressive chunks covering exactly 0..spp-1
        k = 0
        for first, p in passes:
            assert first == k and p >= 1
            k += p
        assert k == res.request.spp


def test_admission_respects_the_budget_and_queues_the_rest():
    ex = FakeExecutor({"a": 10_000})
    step_paths = 1000
    buf = 100 * 100 * 12
    budget = 10_000 + STEPS_IN_FLIGHT * step_paths * PATH_STATE_BYTES + 2 * buf  # room for two 100x100 requests
    srv = RenderServer(ex, budget_bytes=budget, step_paths=step_paths, clock=Clock())
    for i in range(6):
        srv.submit(_req(i, 100, 3))
    srv.step()
    assert len(srv.active) + len(srv.results) <= 2 and len(srv.waiting) >= 4
    while srv.busy():
        srv.step()
        assert srv.resident_bytes() <= budget
    assert ex.peak_live <= 2 and len(srv.results) == 6
    # arrival order is kept for admission
    admitted = sorted(srv.results, key=lambda r: r.admitted)
    assert [r.request.rid for r in admitted] == sorted(r.request.rid for r in admitted)


def test_a_request_too_large_for_the_budget_is_rejected():
    import pytest

    ex = FakeExecutor({"a": 10})
    srv = RenderServer(ex, budget_bytes=1000, step_paths=1, clock=Clock())
    srv.submit(_req(0, 100, 1))
    with pytest.raises(ValueError, match="exceeds the device-memory budget"):
        srv.step()


def test_small_requests_finish_while_a_large_one_continues():
    ex = FakeExecutor({"a": 0})
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=4 * 256 * 256, max_passes_per_step=2, clock=Clock())
    srv.submit(_req(0, 256, 64))
    srv.step()
    srv.submit(_req(1, 32, 2))  # arrives while the large request is in flight
    for _ in range(STEPS_IN_FLIGHT + 1):
        srv.step()
    done = {r.request.rid for r in srv.results}
    assert 1 in done and 0 not in done  # continuous batching: joined and left mid-flight
    assert any(len(items) == 2 for items in ex.steps)  # and shared steps with it


def test_steps_are_pipelined_and_bounded():
    ex = FakeExecutor({"a": 0})
    step_paths = 64 * 64
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=step_paths, min_chunk_paths=0, clock=Clock())
    for i in range(20):
        srv.submit(_req(i, 64, 5))
    for k in range(1, STEPS_IN_FLIGHT):
        srv.step()
        assert ex.pending == k  # launched, not waited for
    srv.step()
    assert ex.pending == STEPS_IN_FLIGHT - 1  # the oldest completed once the pipeline was full
    srv.drain()
    # every step fits in step_paths paths (one wave)
    for items in ex.steps:
        assert sum(p * 64 * 64 for _, _, p in items) <= step_paths
    # round robin: every request was in the first few steps
    first = {rid for items in ex.steps[:20] for rid, _, _ in items}
    assert first == set(range(20))


def test_steps_fill_one_wave_and_never_mix_walk_classes():
    ex = FakeExecutor({"a": 0, "skip": 0})
    step_paths = 100_000
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=step_paths, min_chunk_paths=30_000, clock=Clock())
    sides = [64, 200, 128, 300, 16, 90, 250, 40]
    for i, side in enumerate(sides):
        srv.submit(_req(i, side, 7, "skip" if i % 3 == 0 else "a"))
    srv.submit(_req(99, 400, 2))  # one pass (160,000 paths) is larger than a step
    srv.drain()
    side_of = {i: side for i, side in enumerate(sides)}
    side_of[99] = 400
    cls = {i: (1 if i % 3 == 0 else 0) for i in range(len(sides))}
    cls[99] = 0
    for items in ex.steps:
        paths = sum(p * side_of[rid] ** 2 for rid, _, p in items)
        assert paths <= step_paths or (len(items) == 1 and items[0][2] == 1)
        assert len({cls[rid] for rid, _, _ in items}) == 1
    assert sorted(r.request.rid for r in srv.results) == sorted(list(range(len(sides))) + [99])
    for res in srv.results:
        assert sum(p for _, p in res.image) == res.request.spp


class FailingExecutor(FakeExecutor):
    """Fails the launch of step `bad_launch` and the completion of step `bad_wait` (1-based)."""

    def __init__(self, sb, bad_launch=None, bad_wait=None):
        super().__init__(sb)
        self.bad_launch, self.bad_wait, self.launches = bad_launch, bad_wait, 0

    def launch(self, items):
        self.launches += 1
        if self.launches == self.bad_launch:
            raise RuntimeError("simulated upload failure")
        return super().launch(items)

    def wait(self, ticket):
        super().wait(ticket)
        if ticket == self.bad_wait:
            raise RuntimeError("simulated device error")


@pytest.mark.parametrize("bad_launch,bad_wait", [(2, None), (None, 2), (1, 3)])
def test_a_failed_step_fails_its_requests_and_the_server_goes_on(bad_launch, bad_wait):
    ex = FailingExecutor({"a": 0}, bad_launch, bad_wait)
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=64 * 64 * 2, min_chunk_paths=0, clock=Clock())
    for i in range(8):
        srv.submit(_req(i, 64, 5))
    srv.drain()
    assert sorted(r.request.rid for r in srv.results) == list(range(8))  # every request answered once
    failed = [r for r in srv.results if r.status == "failed"]
    done = [r for r in srv.results if r.status == "done"]
    assert failed and done
    assert all("simulated" in r.error and r.image is None for r in failed)
    for r in done:  # the others got every pass, in order
        assert sum(p for _, p in r.image) == r.request.spp
    assert not ex.live and not srv.active and not srv.inflight  # every buffer released


def test_cancel_waiting_and_in_flight_requests():
    ex = FakeExecutor({"a": 0})
    step_paths = 64 * 64 * 2
    budget = STEPS_IN_FLIGHT * step_paths * PATH_STATE_BYTES + 2 * 64 * 64 * 12  # two requests at a time
    srv = RenderServer(ex, budget_bytes=budget, step_paths=step_paths, min_chunk_paths=0, clock=Clock())
    for i in range(4):
        srv.submit(_req(i, 64, 9))
    srv.step()
    assert {a.req.rid for a in srv.active} == {0, 1}
    assert srv.cancel(3)  # still waiting
    assert srv.cancel(0)  # admitted, passes in flight
    assert not srv.cancel(42)
    srv.drain()
    status = {r.request.rid: r.status for r in srv.results}
    assert status == {0: "cancelled", 1: "done", 2: "done", 3: "cancelled"}
    issued0 = sum(p for items in ex.steps for rid, _, p in items if rid == 0)
    assert issued0 < 9  # no passes launched after the cancel
    assert not any(rid == 3 for items in ex.steps for rid, _, _ in items)
    assert not ex.live


def test_fifo_policy_runs_the_oldest_request_at_full_rate():
    ex = FakeExecutor({"a": 0})
    step_paths = 64 * 64 * 4
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=step_paths, clock=Clock(), policy="fifo")
    srv.submit(_req(0, 64, 12))   # needs three full steps
    srv.submit(_req(1, 16, 4))    # small: fills the leftover room of each wave
    srv.drain()
    steps_with_0 = [items for items in ex.steps if any(rid == 0 for rid, _, _ in items)]
    assert len(steps_with_0) == 3 and all(dict((r, p) for r, _, p in s)[0] == 4 for s in steps_with_0)
    with pytest.raises(ValueError):
        RenderServer(ex, policy="lifo")


def test_srpt_policy_runs_the_request_with_least_work_left_first():
    ex = FakeExecutor({"a": 0})
    step_paths = 64 * 64 * 4
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=step_paths, clock=Clock(), policy="srpt")
    srv.submit(_req(0, 64, 12))   # large, admitted first
    srv.submit(_req(1, 32, 8))    # two steps' worth of a quarter wave each
    srv.submit(_req(2, 16, 4))    # smallest
    results = srv.drain()
    order = [r.request.rid for r in results]
    assert order == [2, 1, 0]
    first = dict((r, p) for r, _, p in ex.steps[0])
    assert first[2] == 4 and first[1] == 8  # the small ones take all they need first
    assert first.get(0, 0) == (step_paths - 16 * 16 * 4 - 32 * 32 * 8) // (64 * 64)
    for r in results:  # every request still gets exactly its passes, in order
        assert [f for f, _ in r.image] == sorted(f for f, _ in r.image)
        assert sum(p for _, p in r.image) == r.request.spp


def test_srpt_age_policy_serves_overdue_requests_first():
    ex = FakeExecutor({"a": 0})
    step_paths = 64 * 64 * 4
    clock = Clock()
    srv = RenderServer(ex, budget_bytes=1 << 40, step_paths=step_paths, clock=clock, policy="srpt_age",
                       age_limit=0.5)
    old = _req(0, 64, 12, arrival=-1.0)   # large and already overdue
    srv.submit(old)
    srv.submit(_req(1, 16, 4, arrival=clock.t + 1.0))  # small and fresh
    srv.step()
    first = dict((r, p) for r, _, p in ex.steps[0])
    assert first[0] == 4  # the overdue request takes the whole step despite its size
    srv.drain()
    assert {r.request.rid for r in srv.results} == {0, 1}
    for r in srv.results:
        assert sum(p for _, p in r.image) == r.request.spp


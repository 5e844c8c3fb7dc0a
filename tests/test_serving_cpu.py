"""Admission policy of the serving loop, on the CPU: a scheduler-only server
(no streams or kernels; launches are recorded) over requests of known sizes."""
import collections
import threading

import numpy as np
import pytest

from smolyax_gb300 import serving


class _Scheduler(serving.Server):
    """Server state without CUDA: request sizes and launch kinds are given,
    launches are recorded instead of run."""

    def __init__(self, budget, n_streams, kinds, bytes_per_point, failing=(), n_fast=0, fast=()):
        self.budget = budget
        self.in_use = 0
        self.streams = ["s%d" % i for i in range(n_streams)]
        self.free_streams = collections.deque(self.streams)
        self.fast_streams = ["f%d" % i for i in range(n_fast)]
        self.free_fast = collections.deque(self.fast_streams)
        self._fast = set(fast)
        self.waiting = collections.deque()
        self.inflight = []
        self.lock = threading.Lock()
        self.completed, self.rejected, self.failed = [], [], []
        self.batch_launches = self.launches = self.admitted = 0
        self.ips = {name: type("IP", (), {"d_in": 3})() for name in kinds}
        self._kinds, self._bpp, self._failing = kinds, bytes_per_point, set(failing)
        self.launched = []

    def request_bytes(self, req):
        return self._bpp[req.name] * req.points

    def _kind(self, req):
        return (req.name in self._fast, self._kinds[req.name])

    def _launch_batch(self, kind, batch, stream, now):
        if any(r.name in self._failing for r, _ in batch):
            raise RuntimeError("the plan cannot serve this request")
        self.launched.append((kind, [r.id for r, _ in batch], stream))


def _req(name, points, op="eval"):
    return serving.Request(name, np.zeros((points, 3)), op=op)


def test_over_budget_request_is_rejected_and_the_rest_served():
    s = _Scheduler(budget=1000, n_streams=4, kinds={"a": None}, bytes_per_point={"a": 10})
    big, small = s.submit(_req("a", 101)), s.submit(_req("a", 5))
    s._admit()
    assert big.error is not None and big.done.is_set() and big in s.rejected
    assert [ids for _, ids, _ in s.launched] == [[small.id]]
    assert s.in_use == 50


def test_requests_wait_in_order_at_the_budget():
    s = _Scheduler(budget=1000, n_streams=8, kinds={"a": None}, bytes_per_point={"a": 10})
    r = [s.submit(_req("a", n)) for n in (60, 30, 20, 5)]
    s._admit()
    # 600 + 300 fit (one merged launch of the same kind); the third (200) does
    # not, and the fourth may not overtake it
    assert [ids for _, ids, _ in s.launched] == [[r[0].id, r[1].id]]
    assert list(s.waiting) == [r[2], r[3]] and s.in_use == 900


def test_merged_launch_per_kind_and_stream_limit():
    s = _Scheduler(budget=10**9, n_streams=2, kinds={"b": "blocked", "c": None, "t": "stream"},
                   bytes_per_point={"b": 1, "c": 1, "t": 1})
    r = [s.submit(_req(n, 10)) for n in ("b", "b", "t", "b", "c")]
    s._admit()
    # two streams: one merged launch of the three 'b' requests, one of 't'; 'c' waits for a stream
    kinds = {k[1]: ids for k, ids, _ in s.launched}
    assert kinds == {"blocked": [r[0].id, r[1].id, r[3].id], "stream": [r[2].id]}
    assert list(s.waiting) == [r[4]] and not s.free_streams


def test_small_requests_take_the_high_priority_streams():
    """Small launches go to the fast streams; when every normal stream is
    busy, a small request behind a waiting large one is still admitted, and
    the large one keeps its place at the head of the queue."""
    s = _Scheduler(budget=10**6, n_streams=1, kinds={"a": None, "b": "x", "f": "blocked"},
                   bytes_per_point={"a": 1, "b": 1, "f": 1}, n_fast=1, fast={"f"})
    a1, b1, f1, f2 = (s.submit(_req(n, 10)) for n in ("a", "b", "f", "f"))
    s._admit()
    got = {k: (ids, st) for k, ids, st in s.launched}
    assert got == {(False, None): ([a1.id], "s0"), (True, "blocked"): ([f1.id, f2.id], "f0")}
    assert list(s.waiting) == [b1] and not s.free_streams and not s.free_fast
    s._release_stream("s0", False)
    s._admit()
    assert s.launched[-1] == ((False, "x"), [b1.id], "s0") and not s.waiting


def test_failed_launch_returns_its_stream_and_memory():
    s = _Scheduler(budget=1000, n_streams=1, kinds={"f": None}, bytes_per_point={"f": 10}, failing={"f"})
    bad = s.submit(_req("f", 10, op="grad"))
    s._admit()
    assert bad.error and bad.done.is_set() and bad in s.failed and s.in_use == 0 and list(s.free_streams) == ["s0"]


def test_failed_merged_launch_fails_every_request_and_returns_everything():
    s = _Scheduler(budget=1000, n_streams=2, kinds={"f": "blocked", "a": None}, bytes_per_point={"f": 10, "a": 1},
                   failing={"f"})
    bad = [s.submit(_req("f", 10)) for _ in range(3)]
    ok = s.submit(_req("a", 10))
    s._admit()
    assert all(r.error and r.done.is_set() and r in s.failed for r in bad)
    assert [ids for _, ids, _ in s.launched] == [[ok.id]]
    assert s.in_use == 10 and len(s.free_streams) == 1  # only the good launch holds memory and a stream


def test_submit_checks_name_and_width():
    s = _Scheduler(budget=1000, n_streams=1, kinds={"a": None}, bytes_per_point={"a": 1})
    with pytest.raises(KeyError):
        s.submit(_req("zz", 1))
    with pytest.raises(ValueError):
        s.submit(serving.Request("a", np.zeros((2, 4))))


def test_pinned_arena_first_fit_and_merging():
    import torch

    from smolyax_gb300.serving import PinnedArena

    a = PinnedArena(4096, pinned=False)  # the allocator logic; page-locking needs a GPU
    x, y, z = a.alloc(1000), a.alloc(256), a.alloc(1)
    assert (x, y, z) == (0, 1024, 1280) and a.in_use == 1536
    assert a.alloc(4096) is None
    a.free(y)
    assert a.alloc(200) == 1024  # first fit reuses the hole
    a.free(x)
    a.free(1024)
    a.free(z)
    assert a.free_list == [(0, 4096)] and a.in_use == 0
    v = a.view(a.alloc(80), (10,), torch.float64)
    v[:] = 3.0
    assert float(v.sum()) == 30.0


def test_launches_on_host_threads_give_back_what_failed_launches_took():
    """With a pool of host threads, launches are prepared there; a launch that
    raises fails its requests and returns its stream and memory, and the
    server is idle once every task has finished."""
    import time
    from concurrent.futures import ThreadPoolExecutor

    s = _Scheduler(budget=1000, n_streams=2, kinds={"f": "blocked", "a": None}, bytes_per_point={"f": 10, "a": 1},
                   failing={"f"})
    s.pool, s.pending, s._building = ThreadPoolExecutor(max_workers=2), 0, {}
    try:
        bad = [s.submit(_req("f", 10)) for _ in range(2)]
        ok = s.submit(_req("a", 10))
        s._admit()
        t0 = time.perf_counter()
        while not s.idle():
            assert time.perf_counter() - t0 < 10
            time.sleep(0.001)
        assert all(r.error and r.done.is_set() for r in bad)
        assert [ids for _, ids, _ in s.launched] == [[ok.id]]
        assert s.in_use == 10 and len(s.free_streams) == 1
    finally:
        s.pool.shutdown(wait=True)

"""Host logic of the plan cache (``_core._PlanCache``) with stand-in plans,
no device: least-recently-used eviction by count and by bytes, closing of
evicted plans under their lock, configuration errors left uncached, a plan
evicted between lookup and use replaced by a fresh one, and one plan shared
by many threads used by one thread at a time."""

from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from ndfiltrs_gb300 import _core


class FakePlan:
    made = 0

    def __init__(self, tag):
        FakePlan.made += 1
        self.tag = tag
        self.open = True
        self.busy = 0
        self.max_busy = 0
        self.lock = threading.Lock()

    @property
    def is_open(self) -> bool:
        return self.open

    def run_host(self, array):
        with self.lock:
            self.busy += 1
            self.max_busy = max(self.max_busy, self.busy)
        time.sleep(0.001)
        with self.lock:
            self.busy -= 1
        return (self.tag, array.sum())

    def close(self) -> None:
        self.open = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def test_eviction_by_count_and_bytes() -> None:
    cache = _core._PlanCache(capacity=3, max_bytes=1 << 30)
    array = np.ones(16, np.float32)
    plans = {}
    for key in "abcd":
        cache.run(key, lambda key=key: plans.setdefault(key, FakePlan(key)), array)
    assert list(cache._plans) == ["b", "c", "d"] and not plans["a"].open
    cache.run("b", lambda: FakePlan("b2"), array)  # a hit: b becomes the most recent
    assert list(cache._plans) == ["c", "d", "b"]
    small = _core._PlanCache(capacity=8, max_bytes=3 * 2 * array.nbytes)
    made = [FakePlan(i) for i in range(5)]
    for i in range(5):
        small.run(i, lambda i=i: made[i], array)
    assert len(small._plans) == 3 and [p.open for p in made] == [False, False, True, True, True]
    small.clear()
    assert not small._plans and not any(p.open for p in made)


def test_errors_are_not_cached() -> None:
    cache = _core._PlanCache()

    def bad():
        raise ValueError("min_count must be between 1 and the number of window elements")

    for _ in range(2):
        with pytest.raises(ValueError):
            cache.run("k", bad, np.ones(4))
    assert not cache._plans


def test_evicted_plan_is_replaced() -> None:
    cache = _core._PlanCache()
    stale = FakePlan("stale")
    cache.run("k", lambda: stale, np.ones(4))
    stale.close()  # closed by another thread's eviction after the lookup
    fresh = []
    result = cache.run("k", lambda: fresh.append(FakePlan("fresh")) or fresh[-1], np.ones(4))
    assert result[0] == "fresh" and not fresh[0].open  # the one-off plan is closed after use


def test_threads_share_one_plan_one_at_a_time() -> None:
    cache = _core._PlanCache()
    made = []
    lock = threading.Lock()

    def make():
        plan = FakePlan("shared")
        with lock:
            made.append(plan)
        return plan

    results = []

    def work():
        results.append(cache.run("k", make, np.ones(8)))

    threads = [threading.Thread(target=work) for _ in range(16)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert len(results) == 16 and all(r[0] == "shared" for r in results)
    assert len(cache._plans) == 1
    cached = cache._plans["k"][0]
    assert cached.open and cached.max_busy == 1
    # Plans made by threads that lost the race to insert are closed.
    assert all(not p.open for p in made if p is not cached)


class SlowPlan(FakePlan):
    """A plan whose filter runs until `release` is set."""

    def __init__(self, tag, started, release):
        super().__init__(tag)
        self.started = started
        self.release = release

    def run_host(self, array):
        self.started.set()
        self.release.wait(10)
        return (self.tag, 0)


def test_evicting_a_busy_plan_does_not_block_other_lookups() -> None:
    """A thread whose insertion evicts a plan that another thread is still
    filtering with waits for that filter outside the cache lock, so lookups
    of unrelated plans go on."""
    cache = _core._PlanCache(capacity=2)
    array = np.ones(4)
    started, release = threading.Event(), threading.Event()
    slow = SlowPlan("slow", started, release)
    cache.run("other", lambda: FakePlan("other"), array)
    filtering = threading.Thread(target=cache.run, args=("slow", lambda: slow, array))
    filtering.start()
    assert started.wait(10)
    cache.run("other", lambda: FakePlan("unused"), array)  # "slow" becomes the least recent
    evicting = threading.Thread(target=cache.run, args=("new", lambda: FakePlan("new"), array))
    evicting.start()
    deadline = time.monotonic() + 10
    while "slow" in cache._plans and time.monotonic() < deadline:
        time.sleep(0.001)
    assert "slow" not in cache._plans
    hit = []
    lookup = threading.Thread(target=lambda: hit.append(cache.run("other", lambda: FakePlan("x"), array)))
    lookup.start()
    lookup.join(2)
    assert hit and hit[0][0] == "other"  # answered while the evicted plan is still busy
    assert slow.open and evicting.is_alive()  # its closer waits for the filter
    release.set()
    filtering.join(10)
    evicting.join(10)
    assert not slow.open

"""Host-side logic of the continuous-batching server, on CPU with a fake
pool: first-fit admission into free slots, HBM-budget rejection,
cancellation, a worker-side exception isolated to its pool, failed cells,
latency statistics.  Failures are injected on the host."""

import heapq

import numpy as np

from pyrometheus_gb300.serving import ReactorServer, Request, latency_stats


class FakePool:
    """Slots whose cells finish after a per-request number of steps."""

    def __init__(self, cap, steps_for=lambda r: 2, fail_step=None,
                 bad_rids=()):
        self.cap = cap
        self.free = list(range(cap))
        heapq.heapify(self.free)
        self.slot_req = np.full(cap, -1)
        self.left = np.zeros(cap, dtype=int)
        self.steps_for = steps_for
        self.fail_step = fail_step
        self.bad = set(bad_rids)
        self.nstep = 0
        self._done = np.zeros(0, dtype=int)
        self.high_water = 0

    def can_admit(self, n):
        return len(self.free) >= n

    def admit(self, r):
        slots = np.array([heapq.heappop(self.free) for _ in range(r.n)])
        self.slot_req[slots] = r.rid
        self.left[slots] = self.steps_for(r)
        return slots

    def release(self, slots):
        for s in slots.tolist():
            heapq.heappush(self.free, s)
        self.slot_req[slots] = -1
        self.left[slots] = 0

    def deactivate(self, slots):
        self.left[slots] = 0

    def reset(self):
        self.__init__(self.cap, self.steps_for)

    def step(self):
        self.nstep += 1
        if self.fail_step is not None and self.nstep == self.fail_step:
            raise RuntimeError("injected worker failure")
        act = self.left > 0
        self.left[act] -= 1
        self._done = np.nonzero(act & (self.left == 0))[0]

    def finished_slots(self):
        d, self._done = self._done, np.zeros(0, dtype=int)
        return d

    def results(self, slots):
        rid = self.slot_req[slots]
        failed = np.array([r in self.bad for r in rid])
        n = len(slots)
        return np.full(n, 1000.0), np.zeros((2, n)), np.ones(n), failed


def req(rid, n, mech="a", arrival=0.0):
    return Request(rid, mech, np.full(n, 1000.0), np.ones((2, n)) / 2,
                   1e5, 1e-3, arrival=arrival)


def drive(server, max_steps=100):
    for _ in range(max_steps):
        if server.idle():
            break
        server.step()


def test_first_fit_admission_and_completion():
    pool = FakePool(10, steps_for=lambda r: 1 + r.rid)
    s = ReactorServer({"a": pool})
    for r in (req(0, 6), req(1, 6), req(2, 3)):
        s.submit(r)
    s.step()
    # 0 and 2 fit (9 slots); 1 waits for free slots
    assert [r.rid for r in s.queue] == [1]
    assert set(s.running) | {r.rid for r in s.done} == {0, 2}
    drive(s)
    assert sorted(r.rid for r in s.done) == [0, 1, 2]
    # 1 was admitted only after 0 freed its slots
    r1 = [r for r in s.done if r.rid == 1][0]
    r0 = [r for r in s.done if r.rid == 0][0]
    assert r1.admitted >= r0.finished
    assert all(r.status == "done" for r in s.done)
    assert pool.can_admit(10)


def test_hbm_budget_rejection_and_cancel():
    pool = FakePool(8, steps_for=lambda r: 5)
    s = ReactorServer({"a": pool})
    big = req(0, 9)
    s.submit(big)
    assert big.status.startswith("rejected") and s.rejected == [big]
    s.submit(req(1, 4))
    s.submit(req(2, 8))          # waits behind 1
    s.step()
    assert s.cancel(2)           # queued
    assert s.cancel(1)           # running: slots are freed
    assert pool.can_admit(8) and s.idle()
    assert {r.status for r in s.done} == {"cancelled"}


def test_worker_exception_is_isolated():
    pa = FakePool(4, steps_for=lambda r: 3, fail_step=2)
    pb = FakePool(4, steps_for=lambda r: 3)
    s = ReactorServer({"a": pa, "b": pb})
    s.submit(req(0, 2, "a"))
    s.submit(req(1, 2, "b"))
    drive(s)
    st = {r.rid: r.status for r in s.done}
    assert st[0].startswith("failed: RuntimeError: injected worker failure")
    assert st[1] == "done"
    # the failed pool serves again afterwards
    s.submit(req(2, 2, "a"))
    drive(s)
    assert s.done[-1].rid == 2 and s.done[-1].status == "done"


def test_failed_cells_mark_request_failed():
    pool = FakePool(4, steps_for=lambda r: 1, bad_rids={0})
    s = ReactorServer({"a": pool})
    s.submit(req(0, 2))
    s.submit(req(1, 2))
    drive(s)
    st = {r.rid: r.status for r in s.done}
    assert st[0].startswith("failed") and st[1] == "done"


def test_run_with_arrivals_and_stats():
    pool = FakePool(16, steps_for=lambda r: 2)
    s = ReactorServer({"a": pool})
    reqs = [req(i, 3, arrival=0.001 * i) for i in range(10)]
    done = s.run(reqs, time_limit=10.0)
    stats = latency_stats(done)
    assert stats["completed"] == 10
    assert stats["p99_ms"] >= stats["p50_ms"] >= 0.0

"""The layout service's scheduling on the CPU: a stand-in batch with a point
budget takes the place of the device batch, so admission order, waiting for
memory, snapshot cadence and retirement are checked without a GPU."""
import types

import numpy as np
import pytest

from graph_gb300 import _abi, serve
from graph_gb300._calls import StatusError


class FakeBatch:
    """Jobs of n points each take n units of a budget; a job runs until its
    tick budget; `add` refuses with CGL_OOM when the budget is short."""

    def __init__(self, device=0, hbm_budget_bytes=0.0):
        self.budget = int(hbm_budget_bytes)
        self.used = 0
        self.jobs = {}
        self.next = 1
        self.added = []
        self.removed = []

    def add(self, positions, links=None, max_ticks=0, stop_below_alpha_min=False, **fields):
        n = len(positions) // 2
        if self.used + n > self.budget:
            raise StatusError("cgl_batch_add", _abi.CGL_OOM)
        job = self.next
        self.next += 1
        self.used += n
        self.jobs[job] = dict(n=n, tick=0, max_ticks=max_ticks, pos=np.asarray(positions, np.float32))
        self.added.append(job)
        return job

    def add_many(self, jobs, threads=0, until_full=False):
        self.calls = getattr(self, "calls", 0) + 1
        ids = []
        for jb in jobs:
            try:
                ids.append(self.add(**jb))
            except StatusError as e:
                if until_full and e.status == _abi.CGL_OOM:
                    return ids
                raise
        return ids

    def remove(self, job):
        self.used -= self.jobs.pop(job)["n"]
        self.removed.append(job)

    def step(self, ticks=1):
        for j in self.jobs.values():
            j["tick"] = min(j["tick"] + ticks, j["max_ticks"])
            j["pos"] = j["pos"] + 1.0

    def state(self, job):
        j = self.jobs[job]
        return types.SimpleNamespace(tick=j["tick"], is_simulation_running=j["tick"] < j["max_ticks"])

    def get_point_positions(self, job):
        return self.jobs[job]["pos"].copy()

    def close(self):
        pass


@pytest.fixture
def service(monkeypatch):
    monkeypatch.setattr(serve, "Batch", FakeBatch)
    ticks = iter(range(10 ** 6))
    snaps = []
    svc = serve.LayoutService(hbm_budget_bytes=100, ticks_per_round=10, snapshot_every=50,
                              on_snapshot=lambda key, tick, pos: snaps.append((key, tick, pos[0])),
                              clock=lambda: float(next(ticks)))
    svc.snaps = snaps
    return svc


def points(n):
    return np.zeros(2 * n, np.float32)


def run_until_idle(svc, limit=1000):
    rounds = 0
    while not svc.idle():
        svc.step_round()
        rounds += 1
        assert rounds < limit
    return rounds


def test_first_come_first_served_and_waiting_for_memory(service):
    # 60 + 30 fit in 100; the third (50) waits at the head of the queue, and the
    # fourth (5), which would fit, waits behind it
    a = service.submit("a", points(60), None, {}, max_ticks=30)
    b = service.submit("b", points(30), None, {}, max_ticks=100)
    c = service.submit("c", points(50), None, {}, max_ticks=20)
    d = service.submit("d", points(5), None, {}, max_ticks=20)
    service.step_round()
    assert [r.key for r in service.running.values()] == ["a", "b"]
    assert [r.key for r in service.queue] == ["c", "d"]
    run_until_idle(service)
    # a retires after 3 rounds; then c and d are admitted (in their order) and retire after 2 more;
    # b after 10
    assert [r.key for r in service.done] == ["a", "c", "d", "b"]
    assert a.finished <= c.admitted <= d.admitted
    assert service.batch.used == 0 and not service.batch.jobs
    for r in (a, b, c, d):
        assert r.ticks == r.max_ticks
        assert r.result is not None


def test_snapshots_every_50_ticks_of_a_job(service):
    r = service.submit("s", points(10), None, {}, max_ticks=120)
    run_until_idle(service)
    assert [(k, t) for k, t, _ in service.snaps] == [("s", 50), ("s", 100)]
    assert r.snapshots == 2
    # the snapshot is the job's positions after that round; the result after the last
    assert [p for _, _, p in service.snaps] == [5.0, 10.0]
    assert r.result[0] == 12.0


def test_retired_jobs_free_their_memory(service):
    for k in range(6):   # 40 points each: two at a time within 100
        service.submit(k, points(40), None, {}, max_ticks=10)
    peak = 0
    while not service.idle():
        service.step_round()
        peak = max(peak, service.batch.used)
    assert peak <= 100
    assert [r.key for r in service.done] == list(range(6))
    assert service.batch.removed == service.batch.added


def test_a_job_that_can_never_fit_is_refused(service):
    service.submit("big", points(150), None, {}, max_ticks=10)
    with pytest.raises(StatusError) as e:
        service.step_round()
    assert e.value.status == _abi.CGL_OOM


def test_a_full_batch_is_not_asked_again_until_a_job_retires(service):
    service.submit("a", points(80), None, {}, max_ticks=30)
    service.submit("b", points(40), None, {}, max_ticks=10)
    service.step_round()                 # a admitted, b refused for memory
    assert service.batch.calls == 1 and len(service.queue) == 1
    service.step_round()                 # nothing retired: no second attempt
    assert service.batch.calls == 1
    service.step_round()                 # a retires at tick 30 ...
    service.step_round()                 # ... and b is admitted on the next round
    assert service.batch.calls == 2 and not service.queue

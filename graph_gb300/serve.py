"""Continuous-batching layout service.

Layout requests arrive over time; each is a graph (positions, links, config)
that runs until alpha < ALPHA_MIN or a tick budget (the animation-frame loop's
end condition, src/index.ts:2164-2169).  The service keeps every admitted job
resident on the device in one `Batch`, advances all of them together a few
ticks per round, admits queued jobs between rounds while the device-memory
budget allows (first come, first served; a refused admission waits until
memory frees up), streams position snapshots every `snapshot_every` ticks of a
job, and retires finished jobs.  Each job's result is the one it would have on
a plain engine of its own.
"""
import collections
import time

from . import _abi
from ._calls import StatusError
from .batch import Batch


class Request:
    __slots__ = ("key", "positions", "links", "fields", "max_ticks", "arrival", "admitted", "finished", "result",
                 "snapshots", "job", "ticks")

    def __init__(self, key, positions, links, fields, max_ticks, arrival):
        self.key = key
        self.positions = positions
        self.links = links
        self.fields = fields
        self.max_ticks = max_ticks
        self.arrival = arrival
        self.admitted = None
        self.finished = None
        self.result = None
        self.snapshots = 0
        self.job = None
        self.ticks = 0


class LayoutService:
    def __init__(self, device=0, hbm_budget_bytes=150e9, ticks_per_round=10, snapshot_every=50,
                 on_snapshot=None, clock=time.perf_counter):
        self.batch = Batch(device=device, hbm_budget_bytes=hbm_budget_bytes)
        self.ticks_per_round = int(ticks_per_round)
        self.snapshot_every = int(snapshot_every)
        self.on_snapshot = on_snapshot
        self.clock = clock
        self.queue = collections.deque()
        self.running = {}
        self.done = []
        self._full = False   # the last admission was refused for memory and no job has retired since

    def submit(self, key, positions, links, fields, max_ticks=1000, arrival=None):
        r = Request(key, positions, links, fields, max_ticks, self.clock() if arrival is None else arrival)
        self.queue.append(r)
        return r

    def _admit(self):
        """Admit queued jobs in arrival order while memory allows: one call for all of them, which
        prepares them (positions, random draws, link lists) on the host's cores at once.  A job
        refused for memory waits, with those behind it, for running jobs to retire (nothing is tried
        again until one has); with none running the refusal is final."""
        if not self.queue or self._full:
            return
        reqs = list(self.queue)
        jobs = [dict(positions=r.positions, links=r.links, max_ticks=r.max_ticks, stop_below_alpha_min=True,
                     **r.fields) for r in reqs]
        ids = self.batch.add_many(jobs, until_full=True)
        if not ids and not self.running:   # the head job alone does not fit: it never will
            raise StatusError("cgl_batch_add_many", _abi.CGL_OOM,
                              "the job at the head of the queue exceeds the device-memory budget")
        self._full = len(ids) < len(reqs)
        now = self.clock()
        for r, job in zip(reqs, ids):
            r.job = job
            r.admitted = now
            self.queue.popleft()
            self.running[job] = r

    def step_round(self):
        """Admit what fits, advance every running job one round, retire finished ones."""
        self._admit()
        if not self.running:
            return 0
        self.batch.step(self.ticks_per_round)
        finished = []
        for job, r in self.running.items():
            s = self.batch.state(job)
            before = r.ticks
            r.ticks = int(s.tick)
            if self.snapshot_every and r.ticks // self.snapshot_every > before // self.snapshot_every:
                r.snapshots += 1
                if self.on_snapshot:
                    self.on_snapshot(r.key, r.ticks, self.batch.get_point_positions(job))
            if not s.is_simulation_running:
                finished.append(job)
        for job in finished:
            r = self.running.pop(job)
            r.result = self.batch.get_point_positions(job)
            r.finished = self.clock()
            self.batch.remove(job)
            self._full = False
            self.done.append(r)
        return len(finished)

    def idle(self):
        return not self.queue and not self.running

    def close(self):
        self.batch.close()

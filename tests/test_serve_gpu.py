"""Continuous-batching service: a job's result is the same alone and in the mix.

Jobs arrive while others are on the GPU; each is admitted between rounds,
advances with the rest, streams snapshots every 50 of its ticks and retires at
its tick budget.  Its final positions must be bit-identical to the same job
on a plain engine of its own, and the snapshots must match the plain engine
at the same tick.
"""
import numpy as np
import pytest

from graph_gb300 import generators

from helpers import same_bits

pytestmark = pytest.mark.gpu


def _job(k):
    n = [300, 1200, 5000, 20000, 800, 3000][k]
    links = generators.preferential_attachment(n, 3, k) if k % 2 else generators.erdos_renyi(n, 6, k)
    space = float(2 ** int(np.clip(np.round(np.log2(41 * np.sqrt(n))), 9, 14)))
    fields = dict(space_size=space, simulation_repulsion=0.1 + 0.05 * k, simulation_link_distance=2.0,
                  random_seed=500 + k)
    return generators.centred_square(n, space, k), links, fields


def _plain(pos, links, fields, ticks, snap_every):
    from graph_gb300.engine import Engine
    e = Engine(**fields)
    e.set_point_positions(pos)
    e.set_links(links)
    e.render()
    e.start(1.0)
    snaps = {}
    for t in range(1, ticks + 1):
        e.step(1)
        if t % snap_every == 0:
            snaps[t] = e.get_point_positions()
    out = e.get_point_positions()
    e.close()
    return out, snaps


def test_jobs_alone_and_in_the_mix():
    from graph_gb300.serve import LayoutService
    snaps = {}
    svc = LayoutService(hbm_budget_bytes=0, ticks_per_round=10, snapshot_every=50,
                        on_snapshot=lambda key, tick, xy: snaps.setdefault(key, {}).__setitem__(tick, xy))
    budgets = [60, 100, 150, 50, 120, 90]
    svc.submit(0, *_job(0), max_ticks=budgets[0])
    svc.submit(1, *_job(1), max_ticks=budgets[1])
    rounds = 0
    while not svc.idle():
        svc.step_round()
        rounds += 1
        if rounds == 2:                      # jobs arrive while others run
            svc.submit(2, *_job(2), max_ticks=budgets[2])
            svc.submit(3, *_job(3), max_ticks=budgets[3])
        if rounds == 5:
            svc.submit(4, *_job(4), max_ticks=budgets[4])
        if rounds == 7:
            svc.submit(5, *_job(5), max_ticks=budgets[5])
    assert len(svc.done) == 6
    for r in svc.done:
        want, want_snaps = _plain(*_job(r.key), budgets[r.key], 50)
        assert r.ticks == budgets[r.key]
        assert same_bits(r.result, want), r.key
        assert sorted(snaps[r.key]) == sorted(want_snaps)
        for t, xy in want_snaps.items():
            assert same_bits(snaps[r.key][t], xy), (r.key, t)
    svc.close()


def test_admission_waits_for_memory():
    from graph_gb300.batch import Batch
    from graph_gb300.serve import LayoutService
    small = _job(0)
    big = _job(3)
    with Batch() as probe:                    # device memory of one big job
        probe.add(big[0], big[1], **big[2])
        one = probe.info().device_bytes
    svc = LayoutService(hbm_budget_bytes=1.5 * one, ticks_per_round=10, snapshot_every=0)
    svc.submit("a", *big, max_ticks=20)
    svc.submit("b", *big, max_ticks=20)      # does not fit beside "a": waits in the queue
    svc.submit("c", *small, max_ticks=20)
    svc.step_round()
    assert len(svc.running) == 1 and len(svc.queue) == 2
    while not svc.idle():
        svc.step_round()
    assert [r.key for r in svc.done][:1] == ["a"] and len(svc.done) == 3
    want, _ = _plain(*big, 20, 1000)
    for r in svc.done:
        if r.key in ("a", "b"):
            assert same_bits(r.result, want)
    svc.close()

"""Batched engine: every job in a batch advances exactly as it would alone.

The reference runs one graph per `Graph`; the batch is an engine extension
whose contract is equivalence: a job's positions after T ticks in a batch are
bit-identical to a plain engine (cgl_create, set positions and links, render,
start(1), step T) with the same config — and so, transitively, to the oracle.
"""
import numpy as np
import pytest

from graph_gb300 import _abi, generators

from helpers import first_mismatch, same_bits

pytestmark = pytest.mark.gpu


def _alone(pos, links, fields, ticks):
    from graph_gb300.engine import Engine
    e = Engine(**fields)
    e.set_point_positions(pos)
    if links is not None:
        e.set_links(links)
    e.render()
    e.start(1.0)
    e.step(ticks)
    out = e.get_point_positions()
    e.close()
    return out


def _jobs(seed=0):
    rng = np.random.default_rng(seed)
    jobs = []
    for k, n in enumerate([1, 2, 3, 40, 150, 600, 2500, 9000, 30000]):
        space = float(2 ** int(np.ceil(np.log2(max(64.0, 40 * np.sqrt(n))))))
        pos = rng.uniform(0, space, size=2 * n).astype(np.float32)
        if k % 2:
            links = generators.barabasi_albert(n, 3, seed + k) if n > 3 else None
        else:
            links = generators.erdos_renyi(n, 6, seed + k) if n > 3 else None
        fields = dict(space_size=space, simulation_repulsion=float(rng.uniform(0.05, 0.5)),
                      simulation_link_distance=2.0, random_seed=1000 + k)
        jobs.append((pos, links, fields))
    # special cases: absent points, a hub list on the side branch, masked stages, no gravity
    pos, links, fields = jobs[6]
    pos = pos.copy()
    pos[10:30] = np.nan
    jobs.append((pos, links, dict(fields, random_seed=77)))
    n = 1200
    star = np.stack([np.zeros(n - 1), np.arange(1, n)], axis=1).astype(np.float32).reshape(-1)
    jobs.append((rng.uniform(500, 1500, size=2 * n).astype(np.float32), star, dict(space_size=2048.0, random_seed=78)))
    jobs.append((jobs[5][0], jobs[5][1], dict(jobs[5][2], stage_mask=_abi.STAGE_MANYBODY | _abi.STAGE_LINK_IN,
                                              random_seed=79)))
    jobs.append((jobs[7][0], jobs[7][1], dict(jobs[7][2], simulation_gravity=0.0, random_seed=80)))
    return jobs


def test_batch_equals_each_job_alone():
    from graph_gb300.batch import Batch
    jobs = _jobs()
    ticks = 12
    with Batch() as b:
        ids = [b.add(pos, links, **fields) for pos, links, fields in jobs]
        info = b.info()
        assert info.jobs == len(jobs)
        b.step(5)
        b.step(ticks - 5)
        many = b.get_positions_many(ids[::-1])[::-1]
        for (pos, links, fields), jid, got2 in zip(jobs, ids, many):
            got = b.get_point_positions(jid)
            want = _alone(pos, links, fields, ticks)
            assert same_bits(got, want), (fields, first_mismatch(got, want))
            assert same_bits(got2, want)
            assert b.state(jid).tick == ticks


def test_tick_budgets_and_alpha_stop():
    from graph_gb300.batch import Batch
    jobs = _jobs(1)[:6]
    with Batch() as b:
        budgets = [3, 7, 0, 11, 5, 9]
        ids = [b.add(pos, links, max_ticks=t, **fields) for (pos, links, fields), t in zip(jobs, budgets)]
        stopper = b.add(jobs[5][0], jobs[5][1], stop_below_alpha_min=True,
                        **dict(jobs[5][2], simulation_decay=3.5, random_seed=5))
        b.step(15)
        for (pos, links, fields), jid, t in zip(jobs, ids, budgets):
            run = t if t else 15
            assert b.state(jid).tick == run
            assert same_bits(b.get_point_positions(jid), _alone(pos, links, fields, run))
        # decay 3.5: alpha is 0.0027 after 3 ticks and 0.00037 after 4, so the loop stops before tick 5
        s = b.state(stopper)
        assert s.tick == 4 and not s.is_simulation_running


def test_jobs_join_and_leave_between_ticks():
    from graph_gb300.batch import Batch
    jobs = _jobs(2)
    with Batch() as b:
        first = [b.add(pos, links, **fields) for pos, links, fields in jobs[:5]]
        b.step(4)
        b.remove(first[1])
        b.remove(first[3])
        later = [b.add(pos, links, **fields) for pos, links, fields in jobs[5:9]]   # reuse freed ranges
        b.step(6)
        for k in (0, 2, 4):
            pos, links, fields = jobs[k]
            assert same_bits(b.get_point_positions(first[k]), _alone(pos, links, fields, 10))
        for (pos, links, fields), jid in zip(jobs[5:9], later):
            assert same_bits(b.get_point_positions(jid), _alone(pos, links, fields, 6))


def _alone_sized(pos, links, fields, ticks, sizes=None):
    from graph_gb300.engine import Engine
    e = Engine(**fields)
    e.set_point_positions(pos)
    if links is not None:
        e.set_links(links)
    if sizes is not None:
        e.set_point_sizes(sizes)
    e.render()
    e.start(1.0)
    e.step(ticks)
    out = e.get_point_positions()
    e.close()
    return out


def test_batch_center_and_collision_equal_alone():
    # ForceCenter and ForceCollision per job, beside jobs without them, in one launch per tick
    from graph_gb300.batch import Batch
    rng = np.random.default_rng(31)
    base = _jobs(3)
    cases = []
    for k, (pos, links, fields) in enumerate(base[3:9]):
        n = pos.size // 2
        sizes = rng.uniform(2, 14, size=n).astype(np.float32) if k % 2 else None
        if sizes is not None:
            sizes[::17] = np.nan                       # NaN -> pointDefaultSize
        extra = [dict(simulation_center=0.4), dict(simulation_collision=0.6),
                 dict(simulation_center=0.3, simulation_collision=0.5, simulation_collision_radius=3.0)][k % 3]
        cases.append((pos, links, dict(fields, **extra, random_seed=500 + k), sizes))
    pos = base[6][0].copy()
    pos[40:80] = np.nan                                # absent points stay out of centroids and grids
    cases.append((pos, base[6][1], dict(base[6][2], simulation_center=0.5, simulation_collision=0.4, random_seed=599),
                  None))
    cases += [(p, l, f, None) for p, l, f in base[:3]]
    ticks = 9
    with Batch() as b:
        ids = [b.add(p, l, sizes=sz, **f) for p, l, f, sz in cases]
        assert b.info().kernels_per_tick > 12
        b.step(ticks)
        for (p, l, f, sz), jid in zip(cases, ids):
            got = b.get_point_positions(jid)
            want = _alone_sized(p, l, f, ticks, sz)
            assert same_bits(got, want), (f, first_mismatch(got, want))


@pytest.mark.parametrize("stream", [_abi.RANDOM_REFERENCE, _abi.RANDOM_COUNTER])
def test_add_many_equals_add(stream):
    from graph_gb300.batch import Batch
    jobs = [(p, l, dict(f, random_stream=stream, device_ingest_min_links=1000.0)) for p, l, f in _jobs(4)]
    with Batch() as one, Batch() as many:
        ids1 = [one.add(p, l, **f) for p, l, f in jobs]
        ids2 = many.add_many([dict(positions=p, links=l, **f) for p, l, f in jobs], threads=4)
        assert len(ids2) == len(jobs)
        one.step(6)
        many.step(6)
        for a, c in zip(ids1, ids2):
            assert same_bits(one.get_point_positions(a), many.get_point_positions(c))
            assert one.state(a).rng_draws == many.state(c).rng_draws


def test_add_many_stops_at_a_bad_job():
    from graph_gb300.batch import Batch
    from graph_gb300._calls import StatusError
    jobs = _jobs(5)[3:7]
    specs = [dict(positions=p, links=l, **f) for p, l, f in jobs]
    specs.insert(2, dict(positions=np.zeros(0, np.float32), links=None, random_seed=1))   # no points
    with Batch() as b:
        with pytest.raises(StatusError):
            b.add_many(specs, threads=3)
        assert b.info().jobs == 2
        b.step(3)
        for jid, (p, l, f) in zip(range(2), jobs[:2]):
            assert same_bits(b.get_point_positions(jid), _alone(p, l, f, 3))


def test_batch_budget_refuses_admission():
    from graph_gb300.batch import Batch
    from graph_gb300._calls import StatusError
    pos = generators.uniform_positions(200_000, 0, 8192, 1)
    with Batch(hbm_budget_bytes=8e6) as b:
        with pytest.raises(StatusError) as ex:
            b.add(pos, None, space_size=8192)
        assert ex.value.status == _abi.CGL_OOM


@pytest.mark.parametrize("dmin", [0.0, float("inf")])
def test_batch_device_and_host_ingest_match_oracle(dmin):
    # the same awkward link set through the batch's device build (0) and host build (inf)
    import math
    from graph_gb300.batch import Batch
    from helpers import make_pair
    rng = np.random.default_rng(9)
    n = 3000
    pos = rng.uniform(0, 4096, size=2 * n).astype(np.float32)
    pos[2 * 5: 2 * 9] = np.nan
    links = generators.erdos_renyi(n, 5, 9).reshape(-1, 2)
    hub = np.stack([np.full(600, 17.0), rng.integers(0, n, 600)], axis=1)
    bad = np.array([[math.nan, 1], [2, -1], [3, n], [4.5, 6], [7, 7], [8, 9], [8, 9]])
    all_links = np.concatenate([links, hub, bad]).astype(np.float32)
    rng.shuffle(all_links)
    all_links = all_links.reshape(-1)
    fields = dict(space_size=4096.0, simulation_repulsion=0.3, simulation_link_distance=2.0, random_seed=91,
                  device_ingest_min_links=dmin)
    with Batch() as b:
        other = b.add(generators.uniform_positions(500, 0, 1024, 3), generators.erdos_renyi(500, 4, 3),
                      space_size=1024.0, random_seed=92, device_ingest_min_links=dmin)
        jid = b.add(pos, all_links, **fields)
        b.step(4)
        got = b.get_point_positions(jid)
    eng, orc = make_pair(pos, all_links, fields)
    orc.step(4)
    want = orc.get_point_positions()
    assert same_bits(got, want), first_mismatch(got, want)


def test_sibling_pairs_in_awkward_jobs():
    # the many-body pass takes two points of one parent cell per thread: cells under 2 units (range
    # flags and the tested re-sums), coincident stacks, a dense job, absent points, odd counts
    from graph_gb300.batch import Batch
    rng = np.random.default_rng(44)
    jobs = []
    pos = rng.uniform(0, 256, size=2 * 20000).astype(np.float32)                 # finest cells 0.5 units
    jobs.append((pos, generators.erdos_renyi(20000, 4, 1), dict(space_size=256.0, random_seed=11)))
    stacks = rng.uniform(100, 900, size=(40, 2))
    pos = stacks[rng.integers(0, 40, 6000)].astype(np.float32).reshape(-1)          # coincident points
    jobs.append((pos, None, dict(space_size=1024.0, random_seed=12)))
    pos = rng.uniform(0, 2048, size=2 * 100000).astype(np.float32)                  # ~0.4 points a cell
    pos[2 * rng.integers(0, 100000, 500)] = np.nan                                  # absent points
    jobs.append((pos, generators.barabasi_albert(100000, 3, 2), dict(space_size=2048.0, random_seed=13)))
    pos = rng.normal(1024, 30, size=2 * 90000).clip(0, 2048).astype(np.float32)    # dense, clustered
    jobs.append((pos, None, dict(space_size=2048.0, random_seed=14, simulation_repulsion=0.7)))
    jobs.append((rng.uniform(0, 512, size=2 * 3).astype(np.float32), None, dict(space_size=512.0, random_seed=15)))
    ticks = 6
    with Batch() as b:
        ids = [b.add(p, l, **f) for p, l, f in jobs]
        b.step(ticks)
        got = b.get_positions_many(ids)
    for (p, l, f), g in zip(jobs, got):
        want = _alone(p, l, f, ticks)
        assert same_bits(g, want), (f, first_mismatch(g, want))

"""Replicas over ranks (graph_gb300/replicas.py) on CPU with gloo, world size 2.

Each rank lays out its share of independent jobs (the oracle stands in for the
engine on CPU); rank 0 gathers every result, and they equal a single-process
run bit for bit.  The timing reductions are the ones bench.py uses under
torchrun.
"""
import os
import socket

import numpy as np
import pytest

from graph_gb300 import generators
from graph_gb300.replicas import assign


def _jobs():
    jobs = []
    for k, n in enumerate([60, 300, 45, 700, 120, 90, 250]):
        pos = generators.uniform_positions(n, 0, 1024, k)
        links = generators.erdos_renyi(n, 4, k)
        jobs.append((pos, links, dict(space_size=1024.0, simulation_repulsion=0.2, random_seed=50 + k)))
    return jobs


def _layout(job):
    from oracle import OracleEngine
    pos, links, fields = job
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.set_links(links)
    o.render()
    o.start(1.0)
    o.step(4)
    out = o.get_point_positions()
    o.close()
    return out


def test_assign_is_balanced_and_complete():
    sizes = [700, 300, 250, 120, 90, 60, 45, 5, 5]
    parts = assign(sizes, 3)
    assert sorted(j for p in parts for j in p) == list(range(len(sizes)))
    loads = [sum(sizes[j] for j in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)
    assert assign(sizes, 3) == parts            # deterministic
    assert assign(sizes, 1) == [list(range(len(sizes)))]


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    from graph_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    jobs = _jobs()
    sizes = [p.size // 2 for p, _, _ in jobs]
    res = replicas.run_jobs(jobs, sizes, _layout)
    slow = replicas.max_over_ranks(1.5 + rank)
    total = replicas.sum_over_ranks(len(replicas.assign(sizes, world)[rank]))
    if rank == 0:
        np.savez(os.path.join(outdir, "res.npz"), *res)
        with open(os.path.join(outdir, "red.txt"), "w") as f:
            f.write("%r %r" % (slow, total))
    else:
        assert res is None
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = np.load(tmp_path / "res.npz")
    want = [_layout(j) for j in _jobs()]
    assert len(got.files) == len(want)
    for k, w in enumerate(want):
        assert np.array_equal(got["arr_%d" % k].view(np.uint32), w.view(np.uint32)), k
    slow, total = open(tmp_path / "red.txt").read().split()
    assert float(slow) == 2.5 and float(total) == len(want)

"""Replicas across GPUs: independent layout jobs partitioned over ranks.

A single graph does not shard cheaply (every stage of a tick ends in a global
dependency), but layout jobs are independent, so N GPUs run N replicas of the
engine, one process per GPU, each on its own share of the jobs, with no
collective on the data path.  Collectives appear only around the timed region
(a barrier and the max of the ranks' times) and to bring results to rank 0.
The same code runs over NCCL on GPUs and over gloo on CPU.
"""
import heapq

import torch
import torch.distributed as dist


def assign(sizes, world):
    """Deterministic longest-first assignment of jobs (by size) to `world` ranks:
    each job goes to the rank with the least work so far (ties to the lower rank).
    Returns one ascending list of job indices per rank."""
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for j in sorted(range(len(sizes)), key=lambda j: (-sizes[j], j)):
        load, r = heapq.heappop(heap)
        out[r].append(j)
        heapq.heappush(heap, (load + sizes[j], r))
    return [sorted(x) for x in out]


def _world():
    if dist.is_available() and dist.is_initialized():
        return dist.get_world_size(), dist.get_rank()
    return 1, 0


def run_jobs(jobs, sizes, runner):
    """Run this rank's share of `jobs` with `runner(job)`; rank 0 returns every
    job's result in job order, other ranks return None."""
    world, rank = _world()
    mine = assign(sizes, world)[rank]
    local = {j: runner(jobs[j]) for j in mine}
    if world == 1:
        return [local[j] for j in range(len(jobs))]
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(local, gathered, dst=0)
    if rank != 0:
        return None
    merged = {}
    for part in gathered:
        merged.update(part)
    return [merged[j] for j in range(len(jobs))]


def max_over_ranks(value, device=None):
    """The largest of the ranks' values (a time: the job ends with the slowest rank)."""
    world, _ = _world()
    if world == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    world, _ = _world()
    if world == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())

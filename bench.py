"""Benchmark: force-layout point-iterations/s on one GB300.

Workload (default): stochastic block model, 1,000,000 points in 200
communities with Zipf(1.2) sizes, mean degree 10 (~5M links, 90% intra),
positions uniform in [0, 8192)^2, spaceSize 8192, repulsion 0.1, gravity 0.25,
friction 0.85, linkSpring 1.0, linkDistance 2.0, decay 5000 — synthetic,
seeded.  One step = one simulation tick (Graph.step()) over the whole graph.

  value  point-iterations/s = live points x ticks / device time, inputs
         resident in HBM, CUDA events on the engine's stream, max over ranks.
  e2e    the same metric through the C ABI with host buffers: each step is
         cgl_step(1) (uploads the tick's alpha and seed, 8 bytes) followed by
         cgl_enqueue_point_positions into pinned host memory (8 bytes per
         point, copied beside the next tick; each call returns once the
         previous tick's copy has landed), timed by the host clock up to the
         last copy (the reference's benchmark story flushes steps with a
         readback, repulsion-benchmark.ts:80-86); e2e.synchronous reads back
         with cgl_get_point_positions after each step instead.
  --impl reference  times the oracle (the CPU restatement of the reference's
         per-tick algorithm; the reference itself is TypeScript/WebGL and
         cannot run here) on all host cores, same workload and metric.

Other workloads (--workload): ba10k (Barabasi-Albert 10,000 points), rmat
(R-MAT scale 23 with collision, --rmat-scale to resize), batch (4,096
independent jobs in one batched engine vs the plain engine job by job), serve
(continuous batching vs a one-job-at-a-time queue under Poisson arrivals),
ingest (Graph.render with the link lists built on the host and on the GPU),
repulsion (the reference's repulsion-benchmark story: 2k-200k points, ms/step).

Multi-GPU (torchrun): replicas only — each rank lays out its own copy of the
graph, no collective on the data path; value = all ranks' points x ticks over
the slowest rank's time (graph_gb300/replicas.py).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _reference_arm(argv):
    for k, a in enumerate(argv):
        if a == "--impl" and k + 1 < len(argv):
            return argv[k + 1] == "reference"
        if a.startswith("--impl="):
            return a.split("=", 1)[1] == "reference"
    return False


# torchrun gives each process OMP_NUM_THREADS=1.  The reference arm runs on
# rank 0 alone, so that rank takes every host core; the count must be set
# before torch or the oracle loads an OpenMP runtime, which reads it once.
def _host_cores():
    # the cores this process may run on (a cgroup or taskset mask can allow fewer than the host has)
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


if _reference_arm(sys.argv[1:]) and int(os.environ.get("WORLD_SIZE", "1")) > 1:
    os.environ["OMP_NUM_THREADS"] = str(_host_cores())

from graph_gb300 import _abi, generators, replicas  # noqa: E402

METRIC = "point-iterations/s"
MANYBODY_NAMES = {0: "one point per thread", 1: "a point over 16 threads", 2: "two points of a cell per thread"}
UNIT = "point-iter/s"


# ------------------------------------------------------------------ workload --
def make_workload(name, seed=1, rmat_scale=23):
    if name == "sbm1m":
        n = 1_000_000
        links = generators.sbm_zipf(n, 200, 1.2, 10, 0.9, seed=seed)
        pos = generators.uniform_positions(n, 0, 8192, seed)
        fields = dict(space_size=8192, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                      simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_decay=5000,
                      random_seed=seed)
        desc = "SBM 1,000,000 points / 200 Zipf(1.2) communities / mean degree 10 / spaceSize 8192"
    elif name == "ba10k":
        n = 10_000
        links = generators.barabasi_albert(n, 5, seed)
        pos = generators.centred_square(n, 4096, seed)
        fields = dict(space_size=4096, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                      simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_decay=5000,
                      random_seed=seed)
        desc = "Barabasi-Albert 10,000 points m=5 / spaceSize 4096"
    elif name == "rmat":
        n = 1 << rmat_scale
        m = 40_000_000 >> (23 - rmat_scale) if rmat_scale <= 23 else 40_000_000 << (rmat_scale - 23)
        links = generators.rmat(rmat_scale, m, 0.57, 0.19, 0.19, seed=seed)
        pos = generators.uniform_positions(n, 0, 16384, seed)
        radius = np.random.default_rng(seed).uniform(1, 8, size=n).astype(np.float32)
        sizes = 2 * radius
        fields = dict(space_size=16384, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                      simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_collision=0.5,
                      simulation_decay=5000, random_seed=seed)
        desc = ("R-MAT scale %d (%s points, a,b,c,d = .57,.19,.19,.05) / %s links / "
                "collision 0.5, radius U[1,8] / spaceSize 16384" % (rmat_scale, format(n, ","), format(m, ",")))
        return pos, links, fields, desc, sizes
    else:
        raise SystemExit("unknown workload %r" % name)
    return pos, links, fields, desc, None


# Algorithmic bytes per launch of each stage (bytes each stage must move at
# minimum; HBM-resident arrays counted once per pass, L2-resident cell data
# counted once per tick in `cells`).  n = live points, m = link entries per
# direction, c = finest cells, cl = cells of all levels.
def stage_bytes(stage, n, m, c, cl):
    return {
        "prepass": 29 * n,          # pos R 8 + flags 1 + pos W 8 + key W 4 + rank W 4 + histogram RMW 4
        "center": 21 * n,
        "scan": 16 * c,             # counts R twice, cell_start W, counts zeroed
        "scatter": 32 * n,          # key 4 + rank 4 + pos 8 + cell_start 4 R; sorted idx 4 + pos 8 W
        "cells": 12 * n + 16 * cl + 8 * c,
        "manybody": 29 * n,         # sorted idx 4 + pos 8, jitter 8, flags 1 R; pos 8 W
        "link_in": 21 * n + 24 * m,  # rowptr 4, own pos 8, flags 1 R, pos 8 W; entry 16 + neighbour pos 8
        "link_out": 21 * n + 24 * m,
        "collision_grid": 13 * n,
        "collision_force": 21 * n,
        "clusters": 54 * n,         # sums: pos 8, cluster 4, flags 1 R (+ K records); pull: pos 8, cluster 4, coeff 4, flags 1 R, pos 8 W
    }[stage]


# The whole tick's algorithmic bytes (the survey's model): gravity, binning,
# scan, many-body and both link passes over N points and E links, the finest
# grid's C_f cells, and with collision its four grids of C_c cells.
def tick_bytes(n, e, cf, cc=None):
    b = 112 * n + 48 * e + 107 * cf
    if cc is not None:
        b += 144 * n + 128 * cc
    return b


def ran_stages(stages, fields):
    """Stage times of the stages that launched work: the engine times every
    stage of the tick, and one whose force is off reads as a short gap."""
    center_on = float(fields.get("simulation_center", 0.0)) != 0.0
    return {k: v for k, v in stages.items() if v > 0 and (k != "center" or center_on)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_ncu(workload):
    """The committed ncu summary of `workload` (profiles/ncu_<workload>.json):
    per kernel stage, per-launch counters of the launches it captured (the
    bench's timed state: ticks 5-7 of the seeded layout), or {}."""
    path = os.path.join(ROOT, "profiles", "ncu_%s.json" % workload)
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


# Launch shares and issue peaks.  An SM issues at most one warp instruction per
# scheduler per cycle: 4 schedulers per SM.
ISSUE_PER_SM_CYCLE = 4


def issue_roofline(dom, dom_ms, ncu, sm_count, sm_mhz, alg_bytes, hbm_peak, hbm_kind):
    """Roofline of an issue-bound kernel: warp instructions per launch (ncu, on
    the benched state) over its event-timed launch, against 4 x SMs x the
    median SM clock of the timed region; the HBM view is kept beside it."""
    k = ncu.get("kernels", {}).get(dom, {})
    inst = k.get("inst_executed")
    peak = ISSUE_PER_SM_CYCLE * sm_count * sm_mhz * 1e6
    achieved = inst / (dom_ms / 1e3) if inst and dom_ms > 0 else None
    hbm = alg_bytes / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    return {"bound": "issue", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "warp-inst/s",
            "frac": achieved / peak if achieved else None, "traffic": k.get("dram_bytes"),
            "launch_ms": dom_ms, "inst_per_launch": inst,
            "peak_source": "architectural: %d issue slots per SM cycle x %d SMs x %.0f MHz (median SM clock of "
                           "the timed region)" % (ISSUE_PER_SM_CYCLE, sm_count, sm_mhz),
            "fp32_pipe_frac_ncu": k.get("fp32_pipe"), "l2_throughput_frac_ncu": k.get("l2_throughput"),
            "issue_active_frac_ncu": k.get("issue_active"),
            "hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
                    "algorithmic_bytes": alg_bytes, "peak_source": hbm_kind},
            "ncu_state": ncu.get("state"), "ncu_source": "profiles/" + ncu.get("file", "")}


def rel_errors(v, ref):
    """Relative error of velocities v against ref (flat x, y pairs): the largest
    and 99th-percentile per-point |dv| / |ref| (points with ref != 0) and the
    norm-wise RMS(|dv|) / RMS(|ref|)."""
    d = np.hypot(v[0::2] - ref[0::2], v[1::2] - ref[1::2])
    r = np.hypot(ref[0::2], ref[1::2])
    ok = r > 0
    q = d[ok] / r[ok]
    return {"max_rel": float(q.max()) if q.size else 0.0, "p99_rel": float(np.percentile(q, 99)) if q.size else 0.0,
            "rms_rel": float(math.sqrt((d * d).mean() / max((r * r).mean(), 1e-300))), "points": int(ok.sum())}


def approximation_error(oracle_engine, tick_note):
    """The many-body velocity of one tick, FP32 (what the engine computes: it is
    bit-exact with the oracle's FP32 restatement) against (1) the same
    grid-pyramid approximation in FP64 at this workload's state and (2) exact
    all-pairs FP64 repulsion at 20,000 points of config 1's density."""
    from oracle import OracleEngine
    v32 = oracle_engine.manybody_velocity(0)
    v64 = oracle_engine.manybody_velocity(1)
    out = {"fp32_vs_fp64_pyramid": dict(rel_errors(v32, v64), state=tick_note)}
    n, space = 20_000, 8192.0
    side = space * math.sqrt(n / 1_000_000)   # 3.8 points per finest cell, as 1M points in 8192^2
    pos = generators.uniform_positions(n, 0, side, 7)
    o = OracleEngine(space_size=space, simulation_repulsion=0.1, random_seed=7)
    o.set_point_positions(pos)
    o.render()
    o.start(1.0)
    exact = o.manybody_velocity(2)
    out["pyramid_vs_exact_20k"] = {
        "fp32": rel_errors(o.manybody_velocity(0), exact),
        "fp64": rel_errors(o.manybody_velocity(1), exact),
        "state": "20,000 points uniform in a %.0f x %.0f square of the 8192 space (config 1's density), tick 0; "
                 "exact = all-pairs FP64 with the same falloff, no jitter" % (side, side)}
    o.close()
    return out


# ------------------------------------------------------------------- clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU side --
def time_oracle(pos, links, fields, budget_s, max_ticks, warmup=1, sizes=None, keep=False):
    """Oracle ticks on all host cores; returns (point-iter/s, ticks timed, seconds, cores[, engine])."""
    from oracle import OracleEngine
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.set_links(links)
    if sizes is not None:
        o.set_point_sizes(sizes)
    o.render()
    o.start(1.0)
    for _ in range(warmup):
        o.step(1)
    t0 = time.perf_counter()
    o.step(1)
    t1 = time.perf_counter() - t0
    ticks = 1
    more = int(min(max_ticks - 1, max(0, budget_s / max(t1, 1e-6) - 1)))
    t0 = time.perf_counter()
    if more > 0:
        o.step(more)
    t = t1 + (time.perf_counter() - t0)
    ticks += max(more, 0)
    live = o.layout().live_points
    cores = int(os.environ.get("OMP_NUM_THREADS", _host_cores()))
    if keep:
        return live * ticks / t, ticks, t, cores, o
    o.close()
    return live * ticks / t, ticks, t, cores


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


# ------------------------------------------------------------------- main --
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sbm1m", choices=["sbm1m", "ba10k", "rmat", "batch", "serve", "ingest", "repulsion"])
    ap.add_argument("--rmat-scale", type=int, default=23, help="R-MAT workload: 2^scale points, 40M * 2^(scale-23) links")
    ap.add_argument("--device-ingest-min", type=float, default=None,
                    help="batched workload: build link lists and jitter on the GPU from this many links/points up")
    ap.add_argument("--rates", default="50,100,200,500,1000,2000", help="request rates (req/s) of the serving sweep")
    ap.add_argument("--requests", type=int, default=200, help="requests per rate of the serving sweep")
    ap.add_argument("--graphs", type=int, default=4096, help="jobs of the batched workload")
    ap.add_argument("--ticks", type=int, default=300, help="ticks per job of the batched workload")
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="time the plain engine on this many jobs only (0 = all) and scale to the whole set")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of oracle ticks for cpu_baseline")
    ap.add_argument("--save-positions", default=None, help="write the final positions (.npy) for profiling runs")
    ap.add_argument("--positions-from", default=None, help="start from saved positions (.npy) instead of the seeded ones")
    ap.add_argument("--quick", action="store_true", help="timed ticks only: no stage profile, e2e or CPU baseline")
    ap.add_argument("--manybody-kernel", default="auto", choices=["auto", "one", "split", "two"],
                    help="the many-body kernel (auto: timed on the first ticks); a profiler's replay distorts "
                         "that timing, so profiled runs name the kernel the unprofiled run keeps")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "ingest":
        run_ingest(args)
        return
    if args.workload == "repulsion":
        run_repulsion(args)
        return

    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    pos, links, fields, desc, sizes = make_workload(args.workload, seed=1 + rank, rmat_scale=args.rmat_scale)
    if args.positions_from:
        pos = np.load(args.positions_from).astype(np.float32)
        desc += " (evolved positions from %s)" % os.path.basename(args.positions_from)
    from graph_gb300.engine import Engine
    kernel = {"auto": _abi.MANYBODY_AUTO, "one": _abi.MANYBODY_ONE_POINT, "split": _abi.MANYBODY_SPLIT,
              "two": _abi.MANYBODY_TWO_POINTS}[args.manybody_kernel]
    eng = Engine(**dict(fields, device=local_rank, manybody_kernel=kernel))
    eng.set_point_positions(pos)
    eng.set_links(links)
    if sizes is not None:
        eng.set_point_sizes(sizes)
    eng.render()
    eng.start(1.0)
    lay = eng.layout()
    live = lay.live_points
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)

    eng.step(args.warmup)
    eng.synchronize()

    clocks = ClockSampler(local_rank)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    eng.step(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    # replicas: every rank lays out its own graph; the job ends with the slowest rank
    ms = replicas.max_over_ranks(ms, device="cuda")
    live_all = replicas.sum_over_ranks(live, device="cuda")
    value = live_all * args.steps / (ms / 1e3)
    tuned = eng.layout()
    mb_kernel = {"kernel": MANYBODY_NAMES.get(int(tuned.manybody_kernel), "?"),
                 "chosen_by": "timing of the first ticks" if tuned.manybody_tuned else
                 ("--manybody-kernel" if args.manybody_kernel != "auto" else "size rule")}
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "steps": args.steps,
                              "ms_per_step": ms / args.steps, "quick": True,
                              "config": {"workload": desc, "manybody_kernel": mb_kernel}}))
        if args.save_positions and rank == 0:
            np.save(args.save_positions, eng.get_point_positions())
        eng.close()
        return

    # per-stage device times (events between the tick's kernels, no graph)
    stages = ran_stages(eng.profile_stages(20), fields)
    m = lay.link_entries_in
    c = lay.finest_grid ** 2
    cl = sum((4 << l) ** 2 for l in range(lay.levels))
    dom = max(stages, key=lambda k: stages[k])
    dom_ms = stages[dom]
    alg = stage_bytes(dom, live, m, c, cl)
    peak, peak_kind = load_peaks()
    achieved = alg / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    ncu = load_ncu(args.workload) if not args.positions_from else {}
    dom_ncu = ncu.get("kernels", {}).get(dom, {})
    sm_count = torch.cuda.get_device_properties(local_rank).multi_processor_count
    sm_mhz = clk.get("sm_mhz") or 2070.0
    if dom == "manybody":
        roofline = issue_roofline(dom, dom_ms, ncu, sm_count, sm_mhz, alg, peak, peak_kind)
    else:
        roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": dom_ncu.get("dram_bytes"), "algorithmic_bytes": alg,
                    "launch_ms": dom_ms, "peak_source": peak_kind}
    per_stage = {k: round(v * 1e3, 2) for k, v in stages.items() if v > 0}
    stage_gbs = {k: round(stage_bytes(k, live, m, c, cl) / (stages[k] / 1e3) / 1e9, 1)
                 for k in stages if stages[k] > 0}
    coll_on = float(fields.get("simulation_collision", 0.0)) != 0.0
    tb = tick_bytes(live, int(lay.links_number), c, int(lay.collision_grid) ** 2 if coll_on else None)
    tick_gbs = tb / (ms / args.steps / 1e3) / 1e9

    # end to end through the C ABI with host buffers: every tick's positions read
    # back into pinned host memory, beside the next tick (two buffers
    # alternate; each call returns once the previous tick's copy has landed),
    # and, for comparison, with the synchronous read-back after each tick
    bufs = [torch.empty(2 * lay.points_number, dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    e2e_steps = max(10, min(args.steps, 200))
    eng.step(1)
    eng.get_point_positions_into(bufs[0])
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        eng.step(1)
        eng.enqueue_point_positions_into(bufs[k & 1])
    eng.synchronize()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0, device="cuda")
    e2e_value = live_all * e2e_steps / e2e_s
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.step(1)
        eng.get_point_positions_into(bufs[0])
    e2e_sync_s = replicas.max_over_ranks(time.perf_counter() - t0, device="cuda")

    cpu = None
    approx = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, ticks, secs, cores, o = time_oracle(pos, links, fields, args.cpu_budget, 50, sizes=sizes, keep=True)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d ticks of the same %s workload on the oracle (C++ restatement, OpenMP, %s), %.1f s"
                         % (ticks, args.workload, cpu_model(), secs)}
        # the oracle as the checker: the approximation error of the tick the engine computes
        approx = approximation_error(o, "tick %d of the seeded layout" % (ticks + 1))
        o.close()

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "points": int(lay.points_number), "links": int(lay.links_number),
                       "link_entries_per_direction": int(m), "finest_grid": int(lay.finest_grid),
                       "levels": int(lay.levels), "step": "one simulation tick (Graph.step)",
                       "l2": "inputs larger than L2 (per-tick working set ~%d MB > 129 MB)"
                             % int((29 * live + 24 * 2 * m + 60 * live) / 1e6),
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "manybody_kernel": mb_kernel},
            "roofline": roofline,
            "tick_roofline": {"bytes_model": "112 N + 48 E + 107 C_f" + (" + 144 N + 128 C_c" if coll_on else ""),
                              "bytes": tb, "achieved": tick_gbs, "peak": peak, "unit": "GB/s",
                              "frac": tick_gbs / peak,
                              "note": "whole tick against HBM; the many-body pass is issue-bound, so the tick "
                                      "sits well below this roof"},
            "stage_us": per_stage,
            "stage_alg_gbs": stage_gbs,
            "cpu_baseline": cpu,
            "approximation_error": approx,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8,
                    "d2h_bytes_per_step": 8 * int(lay.points_number), "steps": e2e_steps,
                    "read_back": "cgl_enqueue_point_positions after each cgl_step: a device copy, then to "
                                 "pinned host memory beside the next tick",
                    "synchronous": {"value": live_all * e2e_steps / e2e_sync_s,
                                    "read_back": "cgl_get_point_positions after each cgl_step"}},
            "gpu_launches": int(lay.kernels_per_tick) * args.steps,
            "clocks": clk,
        }
        print(json.dumps(out))
        if args.save_positions:
            np.save(args.save_positions, eng.get_point_positions())
    eng.close()
    if dist:
        dist.destroy_process_group()


def run_repulsion(args):
    """The reference's own benchmark story (src/stories/performance/
    repulsion-benchmark.ts:13-16, 41-53, 80-88): pure points uniform in a
    4096 space, gravity 0, repulsion 1, decay 1e12, pointDefaultSize 2; per
    size, 12 warm-up steps, a read-back, then 40 steps and a read-back, timed
    by the host clock (ms per step).  The oracle runs the same protocol on the
    host cores beside it (the reference itself needs WebGL)."""
    from graph_gb300.engine import Engine
    from oracle import OracleEngine
    sizes = [2_000, 5_000, 20_000, 50_000, 100_000, 200_000]
    fields = dict(space_size=4096.0, point_default_size=2.0, simulation_decay=1e12, simulation_gravity=0.0,
                  simulation_repulsion=1.0, random_seed=1)
    rows = []
    for n in sizes:
        pos = generators.uniform_positions(n, 0, 4096, n)
        row = {"size": n}
        for name, cls in (("gb300_ms", Engine), ("oracle_ms", OracleEngine)):
            eng = cls(**fields)
            eng.set_point_positions(pos)
            eng.render()
            eng.start(1.0)
            eng.step(12)
            eng.get_point_positions()
            t0 = time.perf_counter()
            eng.step(40)
            eng.get_point_positions()
            row[name] = (time.perf_counter() - t0) * 1e3 / 40
            eng.close()
        row["speedup"] = row["oracle_ms"] / row["gb300_ms"]
        rows.append(row)
    print(json.dumps({"metric": "repulsion benchmark ms/step", "unit": "ms/step", "higher_is_better": False,
                      "n_gpus": 1, "data": "synthetic",
                      "config": {"workload": "repulsion-benchmark story: points only, uniform in 4096^2, gravity 0, "
                                             "repulsion 1, decay 1e12; 12 warm-up + 40 timed steps, read-back "
                                             "flush", "cores_oracle": _host_cores()},
                      "rows": rows}))


def run_ingest(args):
    """Graph.render time (setPointPositions + setLinks applied: positions, jitter,
    both link lists) of the R-MAT graph with the link lists built on the host and
    on the device; the lists are identical (tests/test_device_ingest.py)."""
    import math
    from graph_gb300.engine import Engine
    from graph_gb300 import _abi
    pos, links, fields, desc, sizes = make_workload("rmat", seed=1, rmat_scale=args.rmat_scale)
    out = {}
    for name, dmin in (("host", math.inf), ("device", 0.0)):
        times = []
        for rep in range(max(1, args.steps)):
            eng = Engine(_abi.make_config(**dict(fields, device_ingest_min_links=dmin)))
            eng.set_point_positions(pos)
            eng.set_links(links)
            eng.synchronize()
            t0 = time.perf_counter()
            eng.render()
            eng.synchronize()
            times.append(time.perf_counter() - t0)
            eng.close()
        out[name] = min(times)
    m = links.size // 2
    print(json.dumps({"metric": "links ingested/s", "value": m / out["device"], "unit": "links/s", "n_gpus": 1,
                      "steps": max(1, args.steps), "higher_is_better": True, "data": "synthetic",
                      "config": {"workload": desc, "step": "Graph.render: positions, jitter, both link lists"},
                      "render_s": {"host_build": out["host"], "device_build": out["device"]},
                      "speedup": out["host"] / out["device"]}))


def run_batch(args):
    """Config 3: independent jobs advanced together by the batched engine,
    against the plain engine run job by job on the same GPU.  Both sides do
    the same work per job: ingest (positions, links, render), `ticks` ticks,
    read-back of the final positions."""
    import torch
    from graph_gb300.batch import Batch
    from graph_gb300.engine import Engine
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    jobs = list(generators.batch_workload(args.graphs, seed=7))
    if args.device_ingest_min is not None:
        jobs = [(p, l, dict(f, device_ingest_min_links=args.device_ingest_min)) for p, l, f in jobs]
    gen_s = time.perf_counter() - t0
    n_points = sum(p.size // 2 for p, _, _ in jobs)
    n_links = sum(l.size // 2 for _, l, _ in jobs)
    # batched
    t0 = time.perf_counter()
    b = Batch()
    ids = b.add_many([dict(positions=p, links=l, max_ticks=args.ticks, **f) for p, l, f in jobs])
    b.synchronize()
    t1 = time.perf_counter()
    b.step(args.ticks)
    b.synchronize()
    t2 = time.perf_counter()
    out_batch = b.get_positions_many(ids)
    t3 = time.perf_counter()
    info = b.info()
    batch = {"ingest_s": t1 - t0, "simulate_s": t2 - t1, "readback_s": t3 - t2}
    b.close()
    # plain engine, job by job
    idx = list(range(len(jobs)))
    if args.plain_sample and args.plain_sample < len(jobs):
        rng = np.random.default_rng(11)
        idx = sorted(rng.choice(len(jobs), size=args.plain_sample, replace=False).tolist())
    plain = {"ingest_s": 0.0, "simulate_s": 0.0, "readback_s": 0.0}
    mismatches = 0
    for k in idx:
        p, l, f = jobs[k]
        ta = time.perf_counter()
        e = Engine(**f)
        e.set_point_positions(p)
        e.set_links(l)
        e.render()
        e.start(1.0)
        e.synchronize()
        tb = time.perf_counter()
        e.step(args.ticks)
        e.synchronize()
        tc = time.perf_counter()
        out = e.get_point_positions()
        td = time.perf_counter()
        e.close()
        plain["ingest_s"] += tb - ta
        plain["simulate_s"] += tc - tb
        plain["readback_s"] += td - tc
        a, o = out, out_batch[k]
        same = np.array_equal(np.isnan(a), np.isnan(o)) and np.array_equal(a[~np.isnan(a)].view(np.uint32),
                                                                           o[~np.isnan(o)].view(np.uint32))
        mismatches += 0 if same else 1
    scale = len(jobs) / len(idx)
    plain = {k: v * scale for k, v in plain.items()}
    tot_b = sum(batch.values())
    tot_p = sum(plain.values())
    out = {
        "metric": "batched layouts/s", "value": len(jobs) / tot_b, "unit": "layouts/s",
        "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
        "config": {"workload": "%d jobs, sizes log-uniform [100, 100000], half preferential attachment "
                               "(m 2-6), half Erdos-Renyi (mean degree 4-12), %d ticks each" % (len(jobs), args.ticks),
                   "points": int(n_points), "links": int(n_links), "generate_s": round(gen_s, 1)},
        "batched": dict(batch, layouts_per_s=len(jobs) / tot_b, simulate_layouts_per_s=len(jobs) / batch["simulate_s"],
                        point_iter_per_s=n_points * args.ticks / batch["simulate_s"],
                        kernels_per_tick=int(info.kernels_per_tick), device_gb=info.device_bytes / 1e9),
        "plain": dict(plain, layouts_per_s=len(jobs) / tot_p, simulate_layouts_per_s=len(jobs) / plain["simulate_s"],
                      jobs_timed=len(idx), scaled_to_all=scale != 1.0),
        "speedup_end_to_end": tot_p / tot_b,
        "speedup_simulate": plain["simulate_s"] / batch["simulate_s"],
        "bit_exact_vs_plain": "%d of %d jobs checked identical" % (len(idx) - mismatches, len(idx)),
    }
    print(json.dumps(out))


def serve_requests(count, seed):
    """Config 4 jobs: sizes log-normal (median 5,000 points, sigma 1.5, capped at
    2,000,000), graph type as the batched workload, each until alpha < 0.001 or
    1,000 ticks."""
    rng = np.random.default_rng(seed)
    sizes = np.minimum(2_000_000, np.maximum(2, np.round(np.exp(rng.normal(np.log(5000), 1.5, size=count)))))
    out = []
    for k, n in enumerate(sizes.astype(np.int64)):
        n = int(n)
        gseed = int(rng.integers(0, 2**31))
        if k % 2 == 0:
            links = generators.preferential_attachment(n, int(rng.integers(2, 7)), gseed)
        else:
            links = generators.erdos_renyi(n, float(rng.uniform(4, 12)), gseed)
        space = float(2 ** int(np.clip(np.round(np.log2(41 * np.sqrt(n))), 9, 14)))
        fields = dict(space_size=space, simulation_repulsion=float(rng.uniform(0.05, 0.5)),
                      simulation_link_distance=2.0, simulation_decay=5000, random_seed=gseed)
        out.append((generators.centred_square(n, space, gseed + 1), links, fields))
    return out


def run_serve(args):
    """Config 4: Poisson arrivals at each rate; continuous batching (jobs join
    and leave the device batch between rounds of 10 ticks, snapshots every 50
    ticks, 150 GB admission budget) against a first-come-first-served queue
    that runs one job at a time on a plain engine."""
    import torch
    from graph_gb300.engine import Engine
    from graph_gb300.serve import LayoutService
    torch.cuda.set_device(0)
    jobs = serve_requests(args.requests, seed=9)
    points = sum(p.size // 2 for p, _, _ in jobs)
    max_ticks = 1000
    # plain FIFO: measured service time of each job, then the queue recurrence
    service = []
    for p, l, f in jobs:
        t0 = time.perf_counter()
        e = Engine(**f)
        e.set_point_positions(p)
        e.set_links(l)
        e.render()
        e.start(1.0)
        done = 0
        while done < max_ticks:
            n = e.run(50)
            done += n
            e.get_point_positions()          # the 50-tick snapshot
            if n < 50:
                break
        e.close()
        service.append(time.perf_counter() - t0)
    rows = []
    for rate in [float(r) for r in args.rates.split(",")]:
        rng = np.random.default_rng(int(rate))
        offsets = np.cumsum(rng.exponential(1.0 / rate, size=len(jobs)))
        # FIFO plain engine
        fin, lat = 0.0, []
        for off, st in zip(offsets, service):
            start = max(off, fin)
            fin = start + st
            lat.append(fin - off)
        fifo = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "layouts_per_s": len(jobs) / (fin - offsets[0])}
        # continuous batching, in real time
        svc = LayoutService(hbm_budget_bytes=150e9, ticks_per_round=10, snapshot_every=50)
        t0 = time.perf_counter()
        nxt = 0
        while True:
            now = time.perf_counter() - t0
            while nxt < len(jobs) and offsets[nxt] <= now:
                p, l, f = jobs[nxt]
                svc.submit(nxt, p, l, f, max_ticks=max_ticks, arrival=t0 + offsets[nxt])
                nxt += 1
            if svc.idle():
                if nxt >= len(jobs):
                    break
                time.sleep(max(0.0, offsets[nxt] - (time.perf_counter() - t0)))
                continue
            svc.step_round()
        lat_b = [r.finished - r.arrival for r in svc.done]
        last = max(r.finished for r in svc.done) - t0
        batched = {"p50_s": float(np.percentile(lat_b, 50)), "p99_s": float(np.percentile(lat_b, 99)),
                   "layouts_per_s": len(jobs) / (last - offsets[0]),
                   "snapshots": int(sum(r.snapshots for r in svc.done))}
        svc.close()
        rows.append({"rate_req_s": rate, "batched": batched, "fifo_plain": fifo})
    out = {"metric": "serving p50/p99 time-to-converged-layout and layouts/s", "unit": "s, layouts/s",
           "n_gpus": 1, "data": "synthetic",
           "config": {"requests_per_rate": len(jobs), "points_total": int(points), "max_ticks": max_ticks,
                      "sizes": "log-normal median 5000 sigma 1.5 cap 2,000,000", "round_ticks": 10,
                      "snapshot_every": 50, "budget_gb": 150},
           "plain_service_s": {"mean": float(np.mean(service)), "p50": float(np.percentile(service, 50)),
                               "p99": float(np.percentile(service, 99))},
           "sweep": rows}
    print(json.dumps(out))


def run_reference(args):
    pos, links, fields, desc, sizes = make_workload(args.workload, seed=1, rmat_scale=args.rmat_scale)
    budget = 150.0
    from oracle import OracleEngine
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.set_links(links)
    if sizes is not None:
        o.set_point_sizes(sizes)
    o.render()
    o.start(1.0)
    live = o.layout().live_points
    t0 = time.perf_counter()
    warm = 0
    while warm < args.warmup and (warm == 0 or time.perf_counter() - t0 < budget / 4):
        o.step(1)
        warm += 1
    t_start = time.perf_counter()
    ticks = 0
    while ticks < args.steps:
        o.step(1)
        ticks += 1
        if time.perf_counter() - t_start > budget / 2:
            break
    secs = time.perf_counter() - t_start
    value = live * ticks / secs
    cores = int(os.environ.get("OMP_NUM_THREADS", _host_cores()))
    sample = ("%d of %d requested ticks (after %d warm-up) of the %s workload on the oracle port "
              "(C++ restatement of the reference's per-tick algorithm, OpenMP on %s); the reference itself "
              "is TypeScript + WebGL2 and cannot execute on this machine" % (ticks, args.steps, warm, desc,
                                                                           cpu_model()))
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": ticks, "warmup": warm, "ms_per_step": secs * 1e3 / ticks, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": desc, "step": "one simulation tick (Graph.step)"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    o.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()

"""The paired many-body pass (two points of one finest cell per thread,
graph_gb300/csrc/manybody_duo.cuh) against the oracle, bit for bit.

It runs from 77,824 points with at least one point per finest cell (the finest
grid is capped at 512, so from 262,144 points).  The cases reach each of its
paths: single points at the end of odd cells, dense and coincident cells whose
near-field pairs leave the in-range sequences (a point's cell is then summed
again with the tested chain), level terms without the range flag (finest cell
>= 2 units, every point inside the space), with it (a point pinned outside the
space; cells under 2 units), and quotients outside the reciprocal method's
range (one point at a time).
"""
import numpy as np
import pytest

from graph_gb300 import _abi, generators

from helpers import first_mismatch, make_pair, same_bits

pytestmark = pytest.mark.gpu

N = 300_000


def _positions(kind, space):
    rng = np.random.default_rng(hash(kind) % (1 << 31))
    if kind in ("uniform", "outside_pinned", "tiny_k"):
        return rng.uniform(0, space, size=2 * N).astype(np.float32)
    if kind == "clustered":
        centres = rng.uniform(0.1 * space, 0.9 * space, size=(30, 2))
        pts = centres[rng.integers(0, 30, N)] + rng.normal(0, space / 200, size=(N, 2))
        return np.clip(pts, 0, space).astype(np.float32).reshape(-1)
    if kind == "coincident":
        pos = rng.uniform(0, space, size=(N, 2))
        stacks = rng.uniform(0, space, size=(100, 2))
        k = N // 5
        pos[:k] = stacks[rng.integers(0, 100, k)]
        return pos.astype(np.float32).reshape(-1)
    if kind == "absent":
        pos = rng.uniform(0, space, size=2 * N).astype(np.float32)
        pos[2 * rng.integers(0, N, 5000)] = np.nan
        return pos
    raise KeyError(kind)


CASES = {
    # kind: (space, extra config, many-body only?)
    "uniform": (8192.0, {}, True),
    "clustered": (8192.0, {}, True),
    "coincident": (8192.0, {}, True),
    "absent": (8192.0, {}, True),
    "outside_pinned": (8192.0, {"simulation_gravity": 0.0}, True),
    "small_space": (400.0, {}, True),
    "tiny_k": (8192.0, {"simulation_repulsion": 1e-36}, True),
    "full_tick": (8192.0, {"simulation_link_distance": 2.0}, False),
}


@pytest.mark.parametrize("kind", sorted(CASES))
def test_two_points_per_thread_matches_oracle(kind):
    space, extra, mb_only = CASES[kind]
    pos_kind = "uniform" if kind in ("small_space", "full_tick") else kind
    pos = _positions(pos_kind, space)
    links = generators.erdos_renyi(N, 4, 7) if not mb_only else None
    fields = dict(space_size=space, random_seed=5, manybody_kernel=_abi.MANYBODY_TWO_POINTS, **extra)
    if mb_only:
        fields["stage_mask"] = _abi.STAGE_MANYBODY | (_abi.STAGE_GRAVITY if "simulation_gravity" not in extra else 0)
    pinned = None
    if kind == "outside_pinned":
        pos = pos.copy()
        pos[0:2] = [-50.0, 30.0]            # pinned outside the space: its cell's centroid leaves the cell
        pos[2:4] = [space + 7.0, space / 2]
        pinned = [0, 1]
    eng, orc = make_pair(pos, links, fields, pinned=pinned)
    assert eng.layout().manybody_kernel == _abi.MANYBODY_TWO_POINTS
    for t in range(3):
        eng.step(1)
        orc.step(1)
        a, b = eng.get_point_positions(), orc.get_point_positions()
        assert same_bits(a, b), (kind, t, first_mismatch(a, b))
    ce, co = eng.cells(eng.layout().levels - 1), orc.cells(orc.layout().levels - 1)
    assert same_bits(ce, co)
    assert np.array_equal(eng.slots(), orc.slots())


def test_size_rule_and_tuning():
    # before a graph's first ticks the size rule names the kernel; with
    # CGL_MANYBODY_AUTO the first ticks time the candidates (two ticks each) and
    # keep the fastest; a configured kernel is used as given
    pos = generators.uniform_positions(120_000, 0, 8192, 3)   # 0.46 points per finest cell
    eng, orc = make_pair(pos, None, dict(space_size=8192.0, random_seed=3))
    assert eng.layout().manybody_kernel == _abi.MANYBODY_ONE_POINT
    assert eng.layout().manybody_tuned == 0
    for t in range(7):
        eng.step(1)
        orc.step(1)
        a, b = eng.get_point_positions(), orc.get_point_positions()
        assert same_bits(a, b), (t, first_mismatch(a, b))
    lay = eng.layout()
    assert lay.manybody_tuned == 1
    assert lay.manybody_kernel in (_abi.MANYBODY_ONE_POINT, _abi.MANYBODY_SPLIT)
    small = generators.uniform_positions(5000, 0, 4096, 3)
    e2, _ = make_pair(small, None, dict(random_seed=3))
    assert e2.layout().manybody_kernel == _abi.MANYBODY_SPLIT
    e3, _ = make_pair(small, None, dict(random_seed=3, manybody_kernel=_abi.MANYBODY_TWO_POINTS))
    e3.step(3)
    assert e3.layout().manybody_kernel == _abi.MANYBODY_TWO_POINTS and e3.layout().manybody_tuned == 0


@pytest.mark.parametrize("kind", ["sparse", "dense"])
def test_every_kernel_gives_the_same_layout(kind):
    # the tuner may pick any of the three kernels: each is the same arithmetic
    n = 100_000
    rng = np.random.default_rng(77)
    if kind == "sparse":
        pos = rng.uniform(0, 8192, size=2 * n).astype(np.float32)           # 0.4 points per finest cell
    else:
        pos = rng.normal(4096, 600, size=2 * n).clip(0, 8192).astype(np.float32)
    links = generators.erdos_renyi(n, 4, 77)
    runs = []
    for kernel in (_abi.MANYBODY_ONE_POINT, _abi.MANYBODY_SPLIT, _abi.MANYBODY_TWO_POINTS):
        eng, orc = make_pair(pos, links, dict(space_size=8192.0, random_seed=7, manybody_kernel=kernel))
        eng.step(3)
        assert eng.layout().manybody_kernel == kernel
        runs.append(eng.get_point_positions())
        if kernel == _abi.MANYBODY_ONE_POINT:
            orc.step(3)
            want = orc.get_point_positions()
            assert same_bits(runs[0], want), first_mismatch(runs[0], want)
    for got in runs[1:]:
        assert same_bits(got, runs[0]), first_mismatch(got, runs[0])

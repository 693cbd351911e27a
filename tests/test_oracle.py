"""CPU tests of the parity oracle: known answers, invariants, ingest rules.

The reference ships no tests or golden vectors for this path, so the oracle is
pinned here by (1) published known-answer vectors of the primitives it uses,
(2) invariants stated in the reference's documentation, (3) hand-derived
answers for tiny inputs, and (4) the committed golden fixtures of
tests/golden/ (produced by tests/golden/make_golden.py from first principles).
"""
import json
import math
import os

import numpy as np
import pytest

import oracle
from graph_gb300 import _abi, generators
from oracle import OracleEngine

from seedrandom_ref import SeedRandom
from helpers import mass_seen, scenario

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_splitmix64_published_vector():
    # Vigna's splitmix64.c seeded with 1234567 (the generator's reference output).
    want = [6457827717110365317, 3203168211198807973, 9817491932198370423,
            4593380528125082431, 16408922859458223821]
    assert [oracle.splitmix_draw(1234567, k) for k in range(5)] == want


def test_lowbias32_matches_definition():
    # build-nearfield-slots.vert:130-135, restated independently in numpy
    def ref(h):
        h = np.uint32(h)
        with np.errstate(over="ignore"):
            h ^= h >> np.uint32(16)
            h = np.uint32((int(h) * 0x7FEB352D) & 0xFFFFFFFF)
            h ^= h >> np.uint32(15)
            h = np.uint32((int(h) * 0x846CA68B) & 0xFFFFFFFF)
            h ^= h >> np.uint32(16)
        return int(h)
    rng = np.random.default_rng(3)
    for v in [0, 1, 2, 0xFFFFFFFF, 0x12345678] + list(rng.integers(0, 2**32, size=200)):
        assert oracle.lowbias32(int(v)) == ref(int(v))
    assert oracle.lowbias32(0) == 0


def test_peel_hash_range_and_formula():
    # hashValue = 0.001 + ((h>>8)+0.5)/2^24 * 0.998, f32 (build-nearfield-slots.vert:139-140)
    seed_bits = np.float32(0.37).view(np.uint32)
    for idx in [0, 1, 7, 12345, 2**24 - 1]:
        h = oracle.lowbias32(idx ^ int(seed_bits))
        v = np.float32(np.float32(h >> 8) + np.float32(0.5)) / np.float32(16777216.0)
        want = np.float32(np.float32(0.001) + np.float32(v * np.float32(0.998)))
        got = np.float32(oracle.peel_hash(idx, int(seed_bits)))
        assert got == want
        assert 0.001 <= got < 0.999


def test_cell_index_clamps_like_the_shader():
    assert oracle.cell_index(-5.0, 16.0, 8) == 0
    assert oracle.cell_index(0.0, 16.0, 8) == 0
    assert oracle.cell_index(15.999, 16.0, 8) == 0
    assert oracle.cell_index(16.0, 16.0, 8) == 1
    assert oracle.cell_index(128.0, 16.0, 8) == 7     # p == S clamps into the last cell
    assert oracle.cell_index(1e30, 16.0, 8) == 7
    assert oracle.cell_index(float("nan"), 16.0, 8) == 0


def test_portable_sincos_error_bound():
    # f32 result of an FP64 evaluation: within 1 ulp of the correctly rounded value
    angles = np.float32(np.concatenate([np.arange(0, 5000) * np.float32(0.618033988749895),
                                        np.float32([1e6, 3.3e6, 1e7 - 1, 16777215 * 0.618033988749895])]))
    for a in angles:
        s, c = oracle.sincos(float(a))
        ws, wc = np.float32(math.sin(float(a))), np.float32(math.cos(float(a)))
        for got, want in ((s, ws), (c, wc)):
            ulp = np.spacing(np.float32(abs(want)) if want != 0 else np.float32(1e-30))
            assert abs(np.float32(got) - want) <= ulp, (a, got, want)


def test_rng_draw_order_and_count():
    # jitter: 2 draws per texel of T^2 (ForceManyBody/index.ts:133-138); links:
    # one draw per entry, INCOMING then OUTGOING (ForceLink/index.ts:76,
    # src/index.ts:1663-1666); one peel seed per tick (ForceManyBody/index.ts:521)
    pos, links, fields = scenario("ba_small")
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.set_links(links)
    o.render()
    n = pos.size // 2
    t = math.ceil(math.sqrt(n))
    m = o.layout().link_entries_in
    assert o.state().rng_draws == 2 * t * t + 2 * m
    o.start()
    o.step(7)
    assert o.state().rng_draws == 2 * t * t + 2 * m + 7
    # the first jitter value is draw 0 scaled: float(-1, 1) * 1e-5 of seedrandom(String(seed))
    u0 = SeedRandom(str(fields["random_seed"])).next()
    assert o.jitter()[0] == np.float32((u0 * 2 - 1) * 1e-5)
    # re-setting only the links consumes only link draws
    before = o.state().rng_draws
    o.set_links(links)
    o.render()
    assert o.state().rng_draws == before + 2 * m


def test_csr_matches_adjacency_rules():
    # GraphData._createAdjacencyLists (GraphData/index.ts:525-549) + ForceLink.create
    n = 50
    links = np.array([0, 1, 1, 2, 2, 0, 3, 3, 4, 60, -1, 2, 1.5, 2, 5, 6, 5, 6, np.nan, 1, 0, 2], dtype=np.float32)
    strength = np.array([4, -1, np.inf, 1, 1, 1, 1, 9, 9, 1, 0.25], dtype=np.float32)
    o = OracleEngine(random_seed=5)
    o.set_point_positions(np.zeros(2 * n, dtype=np.float32) + 100)
    o.set_links(links)
    o.set_link_strength(strength)
    o.render()
    pairs = links.reshape(-1, 2)
    valid = [i for i, (s, t) in enumerate(pairs)
             if np.isfinite(s) and np.isfinite(t) and s == int(s) and t == int(t) and 0 <= s < n and 0 <= t < n]
    deg = np.zeros(n)
    for i in valid:
        deg[int(pairs[i][0])] += 1
        deg[int(pairs[i][1])] += 1
    for direction in (0, 1):
        c = o.csr(direction)
        rows = {}
        for i in valid:
            s, t = int(pairs[i][0]), int(pairs[i][1])
            p, q = (s, t) if direction == 0 else (t, s)
            rows.setdefault(p, []).append((q, i))
        at = 0
        for p in range(n):
            assert c["rowptr"][p] == at
            for q, i in rows.get(p, []):
                assert c["col"][at] == q
                dsum = deg[q] + deg[p]
                assert c["bias"][at] == np.float32(deg[q] / dsum if dsum else 0.5)
                si = float(strength[i])
                if not np.isfinite(si) or si < 0:
                    si = 1 / max(min(deg[q], deg[p]), 1)
                assert c["strength"][at] == np.float32(math.sqrt(si))
                at += 1
        assert c["rowptr"][n] == at == len(valid)


def test_alpha_schedule_and_progress():
    # Store.addAlpha: alpha += (0 - alpha) * (1 - 0.001^(1/decay)); progress = sqrt(min(1, 0.001/alpha))
    pos, links, fields = scenario("ba_small")
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.render()
    o.start(1.0)
    o.step(300)
    a = 1.0
    for _ in range(300):
        a += (0 - a) * (1 - math.pow(0.001, 1 / 5000))
    s = o.state()
    assert s.alpha == a
    assert abs(s.alpha - 0.6610) < 1e-3
    assert s.progress == math.sqrt(min(1, 0.001 / a))


def test_run_loop_ends_below_alpha_min():
    o = OracleEngine(random_seed=1, simulation_decay=20)
    o.set_point_positions(generators.uniform_positions(50, 0, 4096, 1))
    o.render()
    o.start(1.0)
    ticks = o.run(100000)
    s = o.state()
    assert s.is_simulation_running == 0 and s.progress == 1.0
    assert s.alpha < 0.001
    # the loop checks alpha before each tick (src/index.ts:2164-2169)
    a, n = 1.0, 0
    while not a < 0.001:
        a += (0 - a) * (1 - math.pow(0.001, 1 / 20))
        n += 1
    assert ticks == n


@pytest.mark.parametrize("kind", ["ba_small", "dense"])
def test_exactly_once_tiling(kind):
    pos, links, fields = scenario(kind)
    fields = dict(fields, stage_mask=_abi.STAGE_MANYBODY)
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.render()
    o.start()
    o.step(1)
    L = o.layout().levels
    cells = [o.cells(l) for l in range(L)]
    seen = mass_seen(cells, pos, fields["space_size"])
    assert np.all(seen == pos.size // 2 - 1)
    for l in range(L):
        assert cells[l][..., 2].sum() == pos.size // 2


def test_sparse_cells_are_exact():
    # docs/many-body-force/README.md:139-144: cells of <= 8 points are sampled
    # exhaustively.  All points inside one 2x2 block of finest cells: the level
    # passes see no mass and the near field equals the all-pairs force times
    # (1 + jitter) (force-nearfield.frag:249).
    rng = np.random.default_rng(7)
    space = 4096.0
    gf = 8   # N=16 -> finest grid 8 (ForceManyBody/index.ts:650-655), cell 512
    # four points in each of the finest cells (1,1), (2,1), (1,2), (2,2)
    blocks = [rng.uniform(520, 1016, size=(4, 2)) + off for off in ([0, 0], [512, 0], [0, 512], [512, 512])]
    pos = np.concatenate(blocks).astype(np.float32).reshape(-1)
    o = OracleEngine(random_seed=3, space_size=space, stage_mask=_abi.STAGE_MANYBODY, simulation_repulsion=1.0)
    o.set_point_positions(pos)
    o.render()
    o.start()
    assert o.layout().finest_grid == gf
    v32 = o.manybody_velocity(0)
    exact = o.manybody_velocity(2)
    jit = o.jitter().astype(np.float64)
    want = exact * (1 + jit)
    cap = 2 * space / gf
    speed = np.hypot(want[0::2], want[1::2])
    assert np.all(speed < cap)
    np.testing.assert_allclose(v32, want, rtol=2e-5, atol=1e-9)


def test_fp64_pyramid_is_close_to_fp32():
    pos, links, fields = scenario("dense")
    o = OracleEngine(**dict(fields, stage_mask=_abi.STAGE_MANYBODY))
    o.set_point_positions(pos)
    o.render()
    o.start()
    v32 = o.manybody_velocity(0)
    v64 = o.manybody_velocity(1)
    scale = np.abs(v64).max()
    assert np.abs(v32 - v64).max() <= 1e-4 * scale


def test_absent_points_are_frozen_and_excluded():
    pos, links, fields = scenario("ba_small")
    pos = pos.copy()
    pos[2 * 5] = np.nan            # half-NaN: the whole point is absent (helper.ts:157-159)
    pos[2 * 9 + 1] = np.nan
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.set_links(links)
    o.render()
    o.start()
    o.step(3)
    p = o.get_point_positions()
    assert np.isnan(p[10:12]).all() and np.isnan(p[18:20]).all()
    assert not np.isnan(np.delete(p, [10, 11, 18, 19])).any()
    assert o.layout().live_points == pos.size // 2 - 2


def test_pinned_points_do_not_move():
    pos, links, fields = scenario("ba_small")
    o = OracleEngine(**fields)
    o.set_point_positions(pos)
    o.set_links(links)
    o.set_pinned_points([3, 4, 1.5, -1, 10 ** 9])
    o.render()
    o.start()
    o.step(5)
    p = o.get_point_positions()
    assert np.array_equal(p[6:10], pos[6:10])
    assert not np.array_equal(p[10:12], pos[10:12])


def test_odd_lengths_warn_and_truncate():
    o = OracleEngine(random_seed=1)
    st = o.set_point_positions(np.array([1, 2, 3, 4, 5], dtype=np.float32))
    assert st == _abi.CGL_WARNING
    st = o.set_links(np.array([0, 1, 1], dtype=np.float32))
    assert st == _abi.CGL_WARNING
    o.render()
    assert o.layout().points_number == 2 and o.layout().links_number == 1


def test_empty_render_is_noop():
    o = OracleEngine(random_seed=1)
    o.render()
    o.start()
    o.step(3)
    assert o.state().tick == 0
    assert o.get_point_positions().size == 0


def test_adjust_space_size():
    o = OracleEngine(random_seed=1, space_size=16384, max_texture_dimension=16384)
    o.set_point_positions(np.full(8, 10000, dtype=np.float32))
    o.render()
    o.start()
    o.step(1)
    assert o.get_point_positions().max() <= 8192     # S reduced to max/2 (Store/index.ts:229-231)


def test_sum_modes_agree_closely():
    # exact cell sums (engine definition) vs sequential f32 blending (reference)
    pos, links, fields = scenario("ba_small")
    out = []
    for mode in (0, 1):
        o = OracleEngine(sum_mode=mode, **fields)
        o.set_point_positions(pos)
        o.set_links(links)
        o.render()
        o.start()
        o.step(5)
        out.append(o.get_point_positions())
    d = np.abs(out[0].astype(np.float64) - out[1])
    assert d.max() < 1e-2


def test_golden_fixtures():
    path = os.path.join(GOLDEN, "golden.json")
    with open(path) as f:
        gold = json.load(f)
    for case in gold["cases"]:
        o = OracleEngine(**case["config"])
        o.set_point_positions(np.array(case["positions"], dtype=np.float32))
        if case.get("links"):
            o.set_links(np.array(case["links"], dtype=np.float32))
        if "clusters" in case:
            o.set_point_clusters(case["clusters"])
        if "cluster_positions" in case:
            o.set_cluster_positions(case["cluster_positions"])
        if "cluster_strength" in case:
            o.set_point_cluster_strength(case["cluster_strength"])
        o.render()
        o.start(1.0)
        o.step(case["ticks"])
        got = o.get_point_positions().astype(np.float64)
        np.testing.assert_allclose(got, np.array(case["expected"]), rtol=0, atol=case["atol"], err_msg=case["name"])


def _rescale_py(pos, space):
    """rescaleInitialNodePositions (Points/index.ts:3134-3218) in Python floats."""
    p = pos.astype(np.float64).reshape(-1, 2)
    live = ~np.isnan(p).any(axis=1)
    if not live.any():
        return pos.copy()
    mnx, mxx = p[live, 0].min(), p[live, 0].max()
    mny, mxy = p[live, 1].min(), p[live, 1].max()
    w, h = mxx - mnx, mxy - mny
    rng = max(w, h)
    out = p.copy()
    if rng == 0:
        c = space / 2
        out[live, 0] = p[live, 0] - mnx + c
        out[live, 1] = p[live, 1] - mny + c
        return out.astype(np.float32).reshape(-1)
    if rng > space:
        return pos.copy()
    n = p.shape[0]
    eff = space * max(1.2, math.sqrt(n) / space) if n > space * space * 0.001 else space * 0.1
    sf = eff / rng
    co = (space - eff) / 2
    ox = ((rng - w) / 2) * sf + co
    oy = ((rng - h) / 2) * sf + co
    out[live, 0] = (p[live, 0] - mnx) * sf + ox
    out[live, 1] = (p[live, 1] - mny) * sf + oy
    return out.astype(np.float32).reshape(-1)


@pytest.mark.parametrize("case", ["sparse", "dense", "one_point", "coincident", "too_wide", "all_absent", "absent"])
def test_rescale_initial_positions(case):
    space = 4096.0
    rng = np.random.default_rng(7)
    if case == "sparse":
        pos = rng.uniform(-50, 80, size=200).astype(np.float32)
    elif case == "dense":   # more points than spaceSize^2 * 0.001
        space = 64.0
        pos = rng.uniform(0, 1, size=2 * 5000).astype(np.float32)
    elif case == "one_point":
        pos = np.array([12.5, -3.0], np.float32)
    elif case == "coincident":
        pos = np.array([7.0, 7.0, 7.0, 7.0, 7.0, 7.0], np.float32)
    elif case == "too_wide":
        pos = np.array([0.0, 0.0, 5000.0, 10.0], np.float32)
    elif case == "all_absent":
        pos = np.array([np.nan, 1.0, 2.0, np.nan], np.float32)
    else:
        pos = rng.uniform(100, 300, size=100).astype(np.float32)
        pos[10] = np.nan
    want = _rescale_py(pos, space)
    o = OracleEngine(random_seed=1, space_size=space, rescale_positions=1, stage_mask=0)
    o.set_point_positions(pos)
    o.render()
    got = o.get_point_positions()
    live = ~(np.isnan(want[0::2]) | np.isnan(want[1::2]))
    assert np.array_equal(np.repeat(live, 2), ~np.isnan(got))
    assert np.array_equal(got[np.repeat(live, 2)], want[np.repeat(live, 2)])


def test_rescale_defaults_and_dont_rescale():
    pos = np.array([1.0, 1.0, 3.0, 2.0], np.float32)
    # rescalePositions undefined: only when the simulation is disabled
    on = OracleEngine(random_seed=1)
    off = OracleEngine(random_seed=1, enable_simulation=0)
    for e in (on, off):
        e.set_point_positions(pos)
        e.render()
    assert np.array_equal(on.get_point_positions(), pos)
    assert not np.array_equal(off.get_point_positions(), pos)
    # dontRescale skips one render's rescale only
    off.set_point_positions_ex(pos, True)
    off.render()
    assert np.array_equal(off.get_point_positions(), pos)
    off.set_point_positions(pos)
    off.render()
    assert not np.array_equal(off.get_point_positions(), pos)


def _collision_cells(xy, grid, cs):
    """Each point's cell in the four offset grids (force-collision-spatial.frag's
    binning, f32 like the shader): an (n, 4, 2) array."""
    xy = xy.reshape(-1, 2).astype(np.float32)
    cs = np.float32(cs)
    out = np.empty((xy.shape[0], 4, 2), dtype=np.int64)
    for g, (ox, oy) in enumerate(((0.0, 0.0), (0.5, 0.0), (0.0, 0.5), (0.5, 0.5))):
        for a, o in ((0, ox), (1, oy)):
            off = xy[:, a] + np.float32(o) * cs
            out[:, g, a] = np.clip(np.floor(off / cs), 0, grid - 1).astype(np.int64)
    return out


def test_collision_result_reads_only_its_windows():
    # The collision pass alone: moving one point changes only the results of the
    # points whose 3x3 window, in one of the four offset grids, holds its old or
    # new cell.  The engine computes every other point's collision result while
    # the longest outgoing hub chains still run, and afterwards computes again
    # only the points in those hubs' windows; this is the property it rests on.
    n = 4000
    rng = np.random.default_rng(5)
    pos = rng.uniform(20, 490, size=2 * n).astype(np.float32)
    sizes = rng.uniform(2, 8, size=n).astype(np.float32)
    fields = dict(space_size=512, simulation_collision=0.7, stage_mask=_abi.STAGE_COLLISION, random_seed=5)

    def one_tick(xy):
        o = OracleEngine(_abi.make_config(**fields))
        o.set_point_positions(xy)
        o.set_point_sizes(sizes)
        o.render()
        o.start(1.0)
        o.step(1)
        return o.get_point_positions(), o.layout()

    late = 17
    moved = pos.copy()
    moved[2 * late:2 * late + 2] = [400.0, 100.0]
    a, lay = one_tick(pos)
    b, _ = one_tick(moved)
    grid, cs = lay.collision_grid, lay.collision_cell_size
    cells = _collision_cells(pos, grid, cs)
    hot = np.concatenate([_collision_cells(pos[2 * late:2 * late + 2], grid, cs),
                          _collision_cells(moved[2 * late:2 * late + 2], grid, cs)])   # (2, 4, 2)
    near = (np.abs(cells[:, None, :, :] - hot[None, :, :, :]) <= 1).all(axis=3)      # (n, 2, 4)
    affected = near.any(axis=(1, 2))
    affected[late] = True
    differ = (a.view(np.uint32).reshape(-1, 2) != b.view(np.uint32).reshape(-1, 2)).any(axis=1)
    assert not (differ & ~affected).any()
    others = affected.copy()
    others[late] = False
    assert (differ & others).any()           # the move does reach the points in its windows
    assert affected.sum() < n // 10

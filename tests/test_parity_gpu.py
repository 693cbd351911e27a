"""GPU parity: the engine's CUDA path against the oracle, through the C ABI.

The bar is bitwise equality of positions after every tick, of every pyramid
level's cells, and of the near-field slots: every FP32 operation is one
correctly rounded IEEE operation in the shaders' order on both sides, and cell
sums are exact, so nothing is left to tolerance.  (The stated tolerance of the
survey, 1e-5 relative per tick, is therefore met with margin 0.)
"""
import math

import numpy as np
import pytest

from graph_gb300 import _abi, generators

from helpers import first_mismatch, make_pair, mass_seen, same_bits, scenario

pytestmark = pytest.mark.gpu


def _assert_same(eng, orc, what=""):
    a, b = eng.get_point_positions(), orc.get_point_positions()
    assert same_bits(a, b), (what, first_mismatch(a, b))


def _assert_cells_and_slots(eng, orc):
    lay = eng.layout()
    for l in range(lay.levels):
        ce, co = eng.cells(l), orc.cells(l)
        assert same_bits(ce, co), ("level", l, first_mismatch(ce, co))
    assert np.array_equal(eng.slots(), orc.slots())


@pytest.mark.parametrize("kind,ticks", [("ba_small", 12), ("dense", 8), ("collision", 5), ("center", 5)])
def test_ticks_bit_exact(kind, ticks):
    pos, links, fields = scenario(kind)
    eng, orc = make_pair(pos, links, fields)
    assert eng.state().rng_draws == orc.state().rng_draws
    for t in range(ticks):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, (kind, "tick", t))
    _assert_cells_and_slots(eng, orc)
    se, so = eng.state(), orc.state()
    assert se.alpha == so.alpha and se.rng_draws == so.rng_draws and se.tick == so.tick


@pytest.mark.parametrize("mask", [_abi.STAGE_GRAVITY, _abi.STAGE_CENTER, _abi.STAGE_MANYBODY, _abi.STAGE_LINK_IN,
                                  _abi.STAGE_LINK_OUT, _abi.STAGE_COLLISION,
                                  _abi.STAGE_GRAVITY | _abi.STAGE_CENTER | _abi.STAGE_MANYBODY])
def test_each_stage_alone(mask):
    pos, links, fields = scenario("collision")
    fields = dict(fields, simulation_center=0.3, stage_mask=mask)
    eng, orc = make_pair(pos, links, fields)
    for t in range(3):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("mask", mask, t))


def test_multi_tick_batches_match_single_steps():
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, fields)
    eng.step(25)             # one call, one parameter upload, 25 graph launches
    for _ in range(25):
        orc.step(1)
    _assert_same(eng, orc)


def test_cfg0_full_run_bit_exact():
    # Barabasi-Albert N=10,000, m=5; 300 ticks
    pos, links, fields = scenario("cfg0")
    eng, orc = make_pair(pos, links, fields)
    eng.step(300)
    orc.step(300)
    _assert_same(eng, orc, "cfg0 after 300 ticks")
    _assert_cells_and_slots(eng, orc)


def test_absent_and_pinned_points():
    pos, links, fields = scenario("ba_small")
    pos = pos.copy()
    pos[2 * 3] = np.nan
    pos[2 * 17 + 1] = np.nan
    pos[2 * 40: 2 * 60] = np.nan
    eng, orc = make_pair(pos, links, fields, pinned=[0, 1, 2, 3, 500, 1999, -4, 2.5])
    for t in range(6):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("tick", t))
    p = eng.get_point_positions()
    assert np.isnan(p[6]) and np.isnan(p[35])
    assert np.array_equal(p[0:6], pos[0:6])
    # pin changes apply immediately (Points/index.ts:1264-1304)
    eng.set_pinned_points(None)
    orc.set_pinned_points(None)
    eng.step(2)
    orc.step(2)
    _assert_same(eng, orc)


def test_collision_with_point_sizes():
    pos, links, fields = scenario("collision")
    sizes = np.random.default_rng(3).uniform(2, 16, size=pos.size // 2).astype(np.float32)
    sizes[::97] = np.nan      # NaN -> pointDefaultSize (GraphData/index.ts:189-194)
    eng, orc = make_pair(pos, links, fields, sizes=sizes)
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("tick", t))
    assert eng.layout().collision_grid == orc.layout().collision_grid


def test_link_strength_and_invalid_links():
    pos, links, fields = scenario("ba_small")
    links = links.copy()
    links[10] = -1
    links[21] = 1e9
    links[33] = 2.5
    links[40] = np.nan
    strength = np.random.default_rng(1).uniform(0, 3, size=links.size // 2).astype(np.float32)
    strength[::13] = -1
    strength[::29] = np.inf
    eng, orc = make_pair(pos, links, fields, strength=strength)
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("tick", t))


@pytest.mark.parametrize("n", [1, 2, 3, 17, 300])
def test_tiny_graphs(n):
    rng = np.random.default_rng(n)
    pos = rng.uniform(0, 4096, size=2 * n).astype(np.float32)
    links = rng.integers(0, n, size=2 * 2 * n).astype(np.float32)
    eng, orc = make_pair(pos, links, dict(random_seed=n))
    for t in range(5):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, (n, t))


def test_hub_lists():
    # a star and a second hub: lists longer than 256 links get a CTA each
    n = 3000
    rng = np.random.default_rng(21)
    pos = rng.uniform(1000, 3000, size=2 * n).astype(np.float32)
    star = np.stack([np.zeros(n - 1), np.arange(1, n)], axis=1)
    hub2 = np.stack([np.arange(2, 900), np.full(898, 1)], axis=1)
    links = np.concatenate([star, hub2, rng.integers(0, n, size=(4000, 2))]).astype(np.float32).reshape(-1)
    eng, orc = make_pair(pos, links, dict(random_seed=21, simulation_link_distance=3.0))
    assert eng.layout().max_degree_in > 256 and eng.layout().max_degree_out > 256
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("hub", t))


def test_hub_lists_with_collision():
    # collision right after the link passes: the outgoing hub chains run on a
    # second stream while the other points' collision sums are taken, and the
    # hubs' points are summed once their chains end
    n = 4000
    rng = np.random.default_rng(23)
    pos = rng.uniform(800, 1300, size=2 * n).astype(np.float32)
    out_star = np.stack([np.zeros(n - 1), np.arange(1, n)], axis=1)          # point 0: a long list each way
    in_star = np.stack([np.arange(2, 1400), np.full(1398, 1)], axis=1)
    links = np.concatenate([out_star, in_star, rng.integers(0, n, size=(6000, 2))]).astype(np.float32).reshape(-1)
    sizes = rng.uniform(2, 10, size=n).astype(np.float32)
    eng, orc = make_pair(pos, links, dict(random_seed=23, simulation_collision=0.6, simulation_link_distance=4.0),
                         sizes=sizes)
    assert eng.layout().max_degree_in > 256 and eng.layout().max_degree_out > 256
    for t in range(5):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("hubs and collision", t))


def test_early_hubs():
    # Incoming lists of 12,000 and 7,000 links (past the leading threshold: at
    # least 4,096 links and half the longest) start their chains beside the
    # many-body pass, after a many-body pass over their points and link
    # targets; a list of 3,000 links stays with the rest of the pass.  The
    # outgoing list of 10,000 links runs on an SM of its own and the one of
    # 4,500 links (under half the longest) on a third stream, both beside the
    # rest of their pass, and the collision results of every other point are
    # computed beside them (their two points sit 1.5 units apart, so their
    # collision windows overlap).  Some targets are absent, some early points
    # pinned (and unpinned later, which uploads the point flags again).
    n = 160_000
    rng = np.random.default_rng(41)
    pos = rng.uniform(500, 3500, size=2 * n).astype(np.float32)
    pos[2 * 50:2 * 60] = np.nan                                                 # absent targets of hub 0
    pos[6:8] = pos[0:2] + 1.5                                                   # outgoing hub 3 beside hub 0
    # the incoming list of point p holds the links (p, q)
    hub0 = np.stack([np.zeros(12_000), np.arange(1, 12_001)], axis=1)
    back0 = np.stack([np.arange(20_000, 30_000), np.zeros(10_000)], axis=1)
    hub1 = np.stack([np.ones(7000), np.arange(30_000, 37_000)], axis=1)
    hub2 = np.stack([np.full(3000, 2), np.arange(40_000, 43_000)], axis=1)
    back3 = np.stack([np.arange(50_000, 54_500), np.full(4500, 3)], axis=1)
    links = np.concatenate([hub0, back0, hub1, hub2, back3, rng.integers(0, n, size=(200_000, 2))])
    links = links.astype(np.float32).reshape(-1)
    sizes = rng.uniform(2, 8, size=n).astype(np.float32)
    fields = dict(random_seed=41, simulation_collision=0.4, simulation_link_distance=3.0, simulation_gravity=0.25)
    eng, orc = make_pair(pos, links, fields, sizes=sizes, pinned=[1, 7, 30_001, 1, 99_999])
    lay = eng.layout()
    assert lay.early_hubs == 2 and 18_985 <= lay.early_points <= 19_010   # 19,002 less the absent targets
    assert lay.leading_out_hubs == 2
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("early hubs", t))
    eng.set_pinned_points([0])
    orc.set_pinned_points([0])
    for t in range(3):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("early hubs, new pins", t))
    _assert_cells_and_slots(eng, orc)
    cfg = _abi.make_config(**dict(fields, simulation_collision=0.0))   # the outgoing pass alone waits for its lead
    eng.set_config(cfg)
    orc.set_config(cfg)
    eng.step(2)
    orc.step(2)
    _assert_same(eng, orc, "leading hubs without collision")
    eng.set_leading_hubs(0)                      # every chain with the rest of its pass again
    assert eng.layout().early_hubs == 0 and eng.layout().leading_out_hubs == 0
    eng.step(2)
    orc.step(2)
    _assert_same(eng, orc, "early hubs off")
    cfg = _abi.make_config(**fields)           # collision again
    eng.set_config(cfg)
    orc.set_config(cfg)
    eng.set_leading_hubs(1, 0)                 # every outgoing chain on the second stream beside the sums
    assert eng.layout().early_hubs == 1 and eng.layout().leading_out_hubs == 0
    eng.step(2)
    orc.step(2)
    _assert_same(eng, orc, "one early hub")
    eng.set_leading_hubs(0, 1)                 # one late point for the collision results
    assert eng.layout().early_hubs == 0 and eng.layout().leading_out_hubs == 1
    eng.step(2)
    orc.step(2)
    _assert_same(eng, orc, "one leading outgoing hub")


def test_springs_outside_the_in_range_sequences():
    # A hub whose list holds neighbours on top of it and well under one unit
    # away, with rest lengths under one unit: springs of length 0 and below 1
    # leave the in-range square root and quotient of the hub chain, so the link
    # pass runs those hub chunks again with the correctly rounded springs.
    n = 1500
    rng = np.random.default_rng(33)
    pos = rng.uniform(1000, 1400, size=2 * n).astype(np.float32)
    pos[2:62] = np.repeat(pos[0:2][None, :], 30, axis=0).reshape(-1)            # 30 points on the hub
    pos[62:262] = (pos[0:2][None, :] + rng.uniform(-0.4, 0.4, size=(100, 2))).reshape(-1).astype(np.float32)
    star = np.stack([np.zeros(n - 1), np.arange(1, n)], axis=1)
    close = rng.integers(1, 131, size=(600, 2))                                  # light rows among them
    links = np.concatenate([star, close]).astype(np.float32).reshape(-1)
    eng, orc = make_pair(pos, links, dict(random_seed=33, simulation_link_distance=0.3))
    assert eng.layout().max_degree_in > 256 or eng.layout().max_degree_out > 256
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("short springs", t))


def test_springs_outside_the_sequences_in_later_chunks():
    # The hub chain runs a chunk while the chunk before it is checked: a chunk
    # that fails its check runs again with the correctly rounded springs, and
    # so does the chunk after it.  Here the failing links sit in a middle chunk
    # and in the last one (the check of the last chunk comes after the chain
    # has ended), and two failing chunks follow each other.  2,399 links: more
    # than the lists whose checks stay on the chain thread.
    n = 2400
    rng = np.random.default_rng(35)
    pos = rng.uniform(1000, 1400, size=2 * n).astype(np.float32)
    hub = pos[0:2].copy()
    for lo, hi in ((700, 712), (900, 906), (1120, 1126), (n - 8, n)):
        pos[2 * lo:2 * hi] = (hub[None, :] + rng.uniform(-0.3, 0.3, size=(hi - lo, 2))).reshape(-1).astype(np.float32)
    pos[2 * 1300:2 * 1302] = np.tile(hub, 2)                                         # on top of the hub
    star = np.stack([np.zeros(n - 1), np.arange(1, n)], axis=1)
    links = np.concatenate([star, rng.integers(1, n, size=(800, 2))]).astype(np.float32).reshape(-1)
    eng, orc = make_pair(pos, links, dict(random_seed=35, simulation_link_distance=0.3))
    assert eng.layout().max_degree_in > 256 or eng.layout().max_degree_out > 256
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("later chunks", t))


def test_level_terms_under_one_unit():
    # Space 32 and a 128-cell finest grid: cells 0.25 units wide, so level
    # centroids within one unit of a point are common and those levels are
    # summed again with the length tested per term.
    n = 3000
    rng = np.random.default_rng(34)
    pos = rng.uniform(0, 32, size=2 * n).astype(np.float32)
    links = generators.erdos_renyi(n, 2, 34)
    eng, orc = make_pair(pos, links, dict(space_size=32.0, random_seed=34, simulation_link_distance=0.5))
    for t in range(3):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("space 32", t))


def test_hub_lists_with_strengths():
    # Hub chunks whose strengths are all 1 leave out the strength product;
    # the star's first 300 links have strength 1 and the rest random ones, so
    # one chain runs both kinds of chunk.
    n = 3000
    rng = np.random.default_rng(22)
    pos = rng.uniform(1000, 3000, size=2 * n).astype(np.float32)
    star = np.stack([np.zeros(n - 1), np.arange(1, n)], axis=1)
    links = np.concatenate([star, rng.integers(0, n, size=(3000, 2))]).astype(np.float32).reshape(-1)
    strength = rng.uniform(0.2, 2.0, size=links.size // 2).astype(np.float32)
    strength[:300] = 1.0
    eng, orc = make_pair(pos, links, dict(random_seed=22, simulation_link_distance=3.0), strength=strength)
    assert max(eng.layout().max_degree_in, eng.layout().max_degree_out) > 256
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("hub strengths", t))


def test_coincident_points_and_outside_space():
    n = 400
    rng = np.random.default_rng(9)
    pos = rng.uniform(-500, 5000, size=2 * n).astype(np.float32)   # some outside [0, S] before the first update
    pos[0:40] = 1234.5                                             # 20 stacked points
    links = generators.erdos_renyi(n, 3, 9)
    for gravity in (0.25, 0.0):
        eng, orc = make_pair(pos, links, dict(random_seed=9, simulation_gravity=gravity, simulation_collision=0.7))
        for t in range(4):
            eng.step(1)
            orc.step(1)
            _assert_same(eng, orc, (gravity, t))


def test_rerender_mid_run():
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, fields)
    eng.step(3)
    orc.step(3)
    new_links = generators.erdos_renyi(pos.size // 2, 4, 77)
    for e in (eng, orc):
        e.set_links(new_links)
        e.render()
    eng.step(3)
    orc.step(3)
    _assert_same(eng, orc, "after setLinks + render")
    new_pos = generators.uniform_positions(2500, 0, 4096, 5)
    for e in (eng, orc):
        e.set_point_positions(new_pos)
        e.render(0.5)
    assert eng.state().rng_draws == orc.state().rng_draws
    eng.step(3)
    orc.step(3)
    _assert_same(eng, orc, "after setPointPositions + render")


def test_config_changes_between_ticks():
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, fields)
    eng.step(2)
    orc.step(2)
    cfg = _abi.make_config(**dict(fields, simulation_repulsion=0.7, simulation_gravity=0.0,
                                  simulation_friction=0.6, simulation_link_distance=5.0))
    eng.set_config(cfg)
    orc.set_config(cfg)
    eng.step(3)
    orc.step(3)
    _assert_same(eng, orc, "after set_config")


def test_run_loop_matches_oracle():
    pos, links, fields = scenario("ba_small")
    fields = dict(fields, simulation_decay=40)
    eng, orc = make_pair(pos, links, fields)
    ne = eng.run(10000)
    no = orc.run(10000)
    assert ne == no > 0
    assert eng.state().is_simulation_running == 0 == orc.state().is_simulation_running
    _assert_same(eng, orc)


def test_exactly_once_tiling_on_gpu():
    pos, links, fields = scenario("dense")
    fields = dict(fields, stage_mask=_abi.STAGE_MANYBODY)
    eng, _ = make_pair(pos, links, fields)
    eng.step(1)
    L = eng.layout().levels
    cells = [eng.cells(l) for l in range(L)]
    seen = mass_seen(cells, pos, fields["space_size"])
    assert np.all(seen == pos.size // 2 - 1)


def test_graph_api_surface():
    from graph_gb300 import Graph
    events = []
    pos, links, fields = scenario("ba_small")
    g = Graph({"spaceSize": 4096, "simulationRepulsion": 0.1, "simulationLinkDistance": 2.0, "randomSeed": 1,
               "simulationDecay": 50,
               "onSimulationStart": lambda: events.append("start"),
               "onSimulationEnd": lambda: events.append("end"),
               "onSimulationPause": lambda: events.append("pause"),
               "onSimulationUnpause": lambda: events.append("unpause")})
    g.setPointPositions(pos)
    g.setLinks(links)
    assert g.getPointPositions().size == 0          # staged until render()
    g.render()
    g.start()
    assert g.isSimulationRunning and g.progress == 0
    g.pause()
    g.step()                                        # step() runs while paused
    g.unpause()
    n = g.run(100000)
    assert n > 0 and not g.isSimulationRunning and g.progress == 1.0
    assert events == ["start", "pause", "unpause", "end"]
    p = g.getPointPositions()
    assert p.size == pos.size and np.isfinite(p).all()
    g.setConfigPartial({"simulationGravity": 0.5})
    assert g.config["simulationGravity"] == 0.5
    g.destroy()
    g.step()                                        # no-op after destroy
    assert g.getPointPositions().size == 0


def _sbm_config1(seed=1):
    # config 1 shape: SBM 1,000,000 points / ~5M links, S = 8192
    n = 1_000_000
    links = generators.sbm_zipf(n, 200, 1.2, 10, 0.9, seed=seed)
    pos = generators.uniform_positions(n, 0, 8192, seed)
    fields = dict(space_size=8192, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                  simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_decay=5000, random_seed=seed)
    return pos, links, fields


def test_sbm_million_ten_ticks_bit_exact():
    # the first 10 ticks: positions after every tick, cells and slots after ticks 1 and 10
    pos, links, fields = _sbm_config1()
    eng, orc = make_pair(pos, links, fields)
    assert eng.state().rng_draws == orc.state().rng_draws
    for t in range(10):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("sbm1M", t))
        if t in (0, 9):
            _assert_cells_and_slots(eng, orc)


def test_sbm_million_full_run_agreement():
    # all 500 ticks of config 1: bit-exact at ticks 250 and 500, agreement figures on record
    from graph_gb300 import agreement
    pos, links, fields = _sbm_config1()
    eng, orc = make_pair(pos, links, fields)
    for block in (250, 250):
        eng.step(block)
        orc.step(block)
        a, b = orc.get_point_positions(), eng.get_point_positions()
        fig = agreement.agreement(a, b, links)
        print("sbm1M tick", eng.state().tick, fig)
        assert fig == dict(procrustes_rms=0.0, procrustes_rms_relative=0.0, edge_length_stress=0.0)
        _assert_same(eng, orc, ("sbm1M tick", eng.state().tick))


def test_full_size_properties():
    # size-independent properties at the benchmark size: determinism across
    # engines, positions inside the space, mass conservation in every level
    n = 1_000_000
    links = generators.sbm_zipf(n, 200, 1.2, 10, 0.9, seed=2)
    pos = generators.uniform_positions(n, 0, 8192, 2)
    fields = dict(space_size=8192, simulation_repulsion=0.1, simulation_link_distance=2.0, random_seed=2)
    from graph_gb300.engine import Engine
    outs = []
    for _ in range(2):
        e = Engine(**fields)
        e.set_point_positions(pos)
        e.set_links(links)
        e.render()
        e.start()
        e.step(20)
        outs.append(e.get_point_positions())
        lay = e.layout()
        for l in range(lay.levels):
            assert e.cells(l)[..., 2].sum() == n
        sl = e.slots()
        fine = e.cells(lay.levels - 1)
        assert np.array_equal((sl >= 0).sum(axis=2), fine[..., 3].astype(np.int64))
        assert np.all(fine[..., 3] == np.minimum(fine[..., 3], np.minimum(8, fine[..., 2])))
        e.close()
    assert same_bits(outs[0], outs[1])
    assert np.all(outs[0] >= 0) and np.all(outs[0] <= 8192)


def test_rmat_scale23_collision_ten_ticks_bit_exact():
    # config 2 shape: R-MAT scale 23 (a,b,c,d = .57,.19,.19,.05), 40M links after
    # self-loop and duplicate removal, radius U[1,8] (pointSizes = 2r), collision
    # 0.5, spaceSize 16384.  Hub lists (up to ~57,000 links) get a CTA each.
    # Positions after each of the first 10 ticks, cells and slots after 1 and 10.
    n = 1 << 23
    links = generators.rmat(23, 40_000_000, 0.57, 0.19, 0.19, seed=3)
    pos = generators.uniform_positions(n, 0, 16384, 3)
    radius = np.random.default_rng(3).uniform(1, 8, size=n).astype(np.float32)
    fields = dict(space_size=16384, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                  simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_collision=0.5,
                  simulation_decay=5000, random_seed=3)
    eng, orc = make_pair(pos, links, fields, sizes=2 * radius)
    assert eng.layout().max_degree_in > 1000 and eng.layout().collision_grid == 0
    assert eng.layout().early_hubs > 0
    for t in range(10):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("rmat23", t))
        if t in (0, 9):
            _assert_cells_and_slots(eng, orc)
    lay = eng.layout()
    assert lay.collision_grid == orc.layout().collision_grid == 512
    orc.close()
    eng.step(3)
    p = eng.get_point_positions()
    assert np.all(p >= 0) and np.all(p <= 16384)
    assert eng.cells(lay.levels - 1)[..., 2].sum() == n


def test_cfg0_late_ticks_bit_exact():
    # config 0 well past its 300 ticks: bit-exact at ticks 300, 600 and 1000
    from graph_gb300 import agreement
    pos, links, fields = scenario("cfg0")
    eng, orc = make_pair(pos, links, fields)
    for block in (300, 300, 400):
        eng.step(block)
        orc.step(block)
        fig = agreement.agreement(orc.get_point_positions(), eng.get_point_positions(), links)
        print("cfg0 tick", eng.state().tick, fig)
        _assert_same(eng, orc, ("cfg0 tick", eng.state().tick))


@pytest.mark.parametrize("mode", ["sim_off_default", "rescale_true", "dont_rescale"])
def test_rescale_positions(mode):
    # Points.updatePositions' rescale (Points/index.ts:390-413, 3134-3218)
    rng = np.random.default_rng(12)
    n = 3000
    pos = rng.uniform(-40, 90, size=2 * n).astype(np.float32)
    pos[2 * 5] = np.nan
    links = generators.erdos_renyi(n, 4, 12)
    from graph_gb300.engine import Engine
    from oracle import OracleEngine
    fields = dict(random_seed=12, space_size=4096)
    if mode == "sim_off_default":
        fields["enable_simulation"] = 0
    else:
        fields["rescale_positions"] = 1
    cfg = _abi.make_config(**fields)
    pair = []
    for cls in (Engine, OracleEngine):
        e = cls(cfg)
        if mode == "dont_rescale":
            e.set_point_positions_ex(pos, True)
        else:
            e.set_point_positions(pos)
        e.set_links(links)
        e.render()
        e.start(1.0)
        pair.append(e)
    eng, orc = pair
    _assert_same(eng, orc, (mode, "render"))
    p = eng.get_point_positions()
    if mode == "dont_rescale":
        assert same_bits(p, np.where(np.isnan(pos.reshape(-1, 2)).any(axis=1, keepdims=True), np.nan,
                                     pos.reshape(-1, 2)).reshape(-1))
    else:
        assert not same_bits(p, pos) and np.nanmin(p) >= 0 and np.nanmax(p) <= 4096
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, (mode, t))


@pytest.mark.parametrize("stream", [_abi.RANDOM_REFERENCE, _abi.RANDOM_COUNTER])
def test_random_streams_match_oracle(stream):
    # both streams: jitter and link draws (on the device for the counter
    # stream, from the host for the reference's), then a few ticks
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, dict(fields, random_stream=stream, device_ingest_min_links=0.0))
    assert eng.state().rng_draws == orc.state().rng_draws
    for t in range(4):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, (stream, t))


def test_string_seed_matches_oracle():
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, dict(fields, random_seed="layout-α"))
    for t in range(3):
        eng.step(1)
        orc.step(1)
        _assert_same(eng, orc, ("string seed", t))


def test_binning_order_switches():
    # From the second tick the pass bins in the previous tick's cell order; a
    # tick with the center force bins in point order (its centroid pass does
    # the binning), a render of new positions starts over in point order, and
    # pin changes apply in either order.
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, dict(fields, simulation_gravity=0.2))
    plan = [({}, 2), ({"simulation_center": 0.4}, 2), ({}, 2), ("pin", 2), ("render", 3), ({"simulation_gravity": 0.0}, 2)]
    base = dict(fields, simulation_gravity=0.2)
    for change, ticks in plan:
        if change == "pin":
            for e in (eng, orc):
                e.set_pinned_points([1, 5, 9, 300])
        elif change == "render":
            new_pos = generators.uniform_positions(pos.size // 2, 100, 4000, 8)
            for e in (eng, orc):
                e.set_point_positions(new_pos)
                e.render()
        else:
            cfg = _abi.make_config(**dict(base, **change))
            eng.set_config(cfg)
            orc.set_config(cfg)
        for t in range(ticks):
            eng.step(1)
            orc.step(1)
            _assert_same(eng, orc, (change, t))
    _assert_cells_and_slots(eng, orc)

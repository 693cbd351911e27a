"""Pointer interaction: right-click repulsion (force-mouse.frag), drag
(drag-point.frag) and the animation-frame loop (src/index.ts:2152-2317).

CPU tests pin the oracle with hand-computed values; GPU tests hold the engine
to bitwise equality with the oracle through frames, steps and runs.
"""
import numpy as np
import pytest

from graph_gb300 import _abi

from helpers import first_mismatch, make_pair, same_bits, scenario

MOUSE = dict(enable_right_click_repulsion=1)


def _oracle(fields, pos):
    from oracle import OracleEngine
    o = OracleEngine(**fields)
    o.set_point_positions(np.asarray(pos, dtype=np.float32))
    o.render()
    return o


def test_mouse_push_by_hand():
    # point (100, 100), pointer (100, 50): d = (0, -50), |d| = 50 -> 100 * 2 / 2500 = 0.08
    # along -(0, -1): v = (0, 0.08), times friction 0.85
    o = _oracle(dict(random_seed=1, stage_mask=0, **MOUSE), [100.0, 100.0, 3000.0, 3000.0])
    o.start(1.0)
    o.set_pointer(100.0, 50.0, True)
    o.step(1)
    p = o.get_point_positions()
    assert p[0] == 100.0 and p[1] == np.float32(np.float32(100.0) + np.float32(np.float32(0.08) * np.float32(0.85)))
    assert o.state().alpha >= 0.1


def test_mouse_close_range_and_coincident():
    # |d| < 10 uses 10: 100 * 2 / 100 = 2; the pointer on the point pushes along +x
    o = _oracle(dict(random_seed=1, stage_mask=0, simulation_friction=1.0, **MOUSE), [500.0, 500.0, 600.0, 503.0])
    o.start(1.0)
    o.set_pointer(500.0, 500.0, True)
    o.step(1)
    p = o.get_point_positions()
    assert p[0] == 498.0 and p[1] == 500.0                      # direction (1, 0), pushed by -2
    assert np.isclose(p[2], 600.0 + 200.0 / (100.0 ** 2 + 9.0) * 100.0 / np.hypot(100.0, 3.0), rtol=1e-6)


def test_mouse_needs_config_and_button():
    pos = [100.0, 100.0, 300.0, 300.0]
    a = _oracle(dict(random_seed=1, stage_mask=0), pos)            # repulsion not enabled
    a.start(1.0)
    a.set_pointer(100.0, 50.0, True)
    a.step(1)
    b = _oracle(dict(random_seed=1, stage_mask=0, **MOUSE), pos)   # button not held
    b.start(1.0)
    b.set_pointer(100.0, 50.0, False)
    b.step(1)
    assert np.array_equal(a.get_point_positions(), np.float32(pos))
    assert np.array_equal(b.get_point_positions(), np.float32(pos))


def test_frames_when_paused_still_push_and_drag():
    pos = [100.0, 100.0, 300.0, 300.0, 900.0, 900.0]
    o = _oracle(dict(random_seed=1, enable_drag=1, **MOUSE), pos)
    o.start(1.0)
    o.pause()
    o.set_pointer(310.0, 290.0, True)
    assert o.frame(2) == 0                          # no tick while paused
    p = o.get_point_positions()
    assert p[0] != 100.0                            # but the pointer pass ran
    o.set_pointer(1234.5, 777.25, False)
    o.set_drag(2)
    o.frame(1)
    p = o.get_point_positions()
    assert p[4] == 1234.5 and p[5] == 777.25
    o.set_drag(None)
    o.set_pointer(5.0, 5.0, False)
    o.frame(1)
    assert o.get_point_positions()[4] == 1234.5


def test_drag_ignored_without_enable_drag():
    o = _oracle(dict(random_seed=1), [100.0, 100.0, 300.0, 300.0])
    o.start(1.0)
    o.pause()
    o.set_pointer(50.0, 60.0, False)
    o.set_drag(1)
    o.frame(1)
    assert o.get_point_positions()[2] == 300.0


def test_frame_loop_ends_simulation():
    o = _oracle(dict(random_seed=1, simulation_decay=2.0, stage_mask=0), [100.0, 100.0, 300.0, 300.0])
    o.start(1.0)
    ticks = o.frame(100)
    assert 0 < ticks < 100 and not o.state().is_simulation_running and o.state().progress == 1.0


# ----------------------------------------------------------------------- GPU --
def _same(eng, orc, what):
    a, b = eng.get_point_positions(), orc.get_point_positions()
    assert same_bits(a, b), (what, first_mismatch(a, b))
    assert eng.state().alpha == orc.state().alpha and eng.state().tick == orc.state().tick


@pytest.mark.gpu
def test_mouse_and_drag_bit_exact():
    pos, links, fields = scenario("ba_small")
    eng, orc = make_pair(pos, links, dict(fields, enable_drag=1, **MOUSE), pinned=[7])
    for e in (eng, orc):
        e.set_pointer(2048.0, 2000.0, True)
    for t in range(3):
        eng.step(1)
        orc.step(1)
        _same(eng, orc, ("step", t))
    for e in (eng, orc):
        e.set_pointer(1800.5, 2100.25, True)
        e.set_drag(7)                      # a pinned point follows the pointer too
    assert eng.frame(4) == orc.frame(4) == 4
    _same(eng, orc, "frames")
    for e in (eng, orc):
        e.pause()
    assert eng.frame(3) == orc.frame(3) == 0
    _same(eng, orc, "paused frames")
    for e in (eng, orc):
        e.unpause()
        e.set_pointer(100.0, 100.0, False)
    assert eng.run(5) == orc.run(5) == 5
    _same(eng, orc, "run with drag")
    for e in (eng, orc):
        e.set_drag(None)
    assert eng.frame(6) == orc.frame(6) == 6   # no interaction: the fast path
    _same(eng, orc, "plain frames")


@pytest.mark.gpu
def test_frame_loop_end_matches():
    pos, links, fields = scenario("center")
    eng, orc = make_pair(pos, links, dict(fields, simulation_decay=20.0))
    n1, n2 = eng.frame(400), orc.frame(400)
    assert n1 == n2 < 400 and not eng.state().is_simulation_running
    _same(eng, orc, "ended")


@pytest.mark.gpu
def test_graph_surface_clusters_pointer_texture():
    # clusters, the pointer and the position texture through the camelCase Graph
    from graph_gb300 import Graph, generators
    n = 2000
    pos = generators.uniform_positions(n, 1000, 3000, 4)
    links = generators.erdos_renyi(n, 4, 4)
    clusters = [k % 3 if k % 7 else None for k in range(n)]
    events = []
    g = Graph({"spaceSize": 4096, "simulationCluster": 0.3, "enableDrag": True, "enableRightClickRepulsion": True,
               "simulationRepulsionFromMouse": 2, "randomSeed": 3,
               "onDragStart": lambda: events.append("drag"), "onDragEnd": lambda: events.append("drop")})
    g.setPointPositions(pos)
    g.setLinks(links)
    g.setPointClusters(clusters)
    g.setClusterPositions([500, 600, None, None])
    g.render()
    g.start()
    g.setPointer(1200.0, 900.0, rightButton=True)
    g.startDrag(3)
    assert g.frame(5) == 5
    p = g.getPointPositions()
    assert p[6] == np.float32(1200.0) and p[7] == np.float32(900.0)   # the dragged point sits on the pointer
    g.endDrag()
    assert events == ["drag", "drop"]
    tex = g.getPositionTexture()
    t = int(np.ceil(np.sqrt(n)))
    assert tex.shape == (t * t, 4)
    assert np.array_equal(tex[:n, 0], p[0::2]) and np.array_equal(tex[:n, 2], np.arange(n, dtype=np.float32))
    assert not tex[n:].any()
    c = g.getClusterPositions()
    assert c.size == 6 and np.isfinite(c).all()
    g.destroy()

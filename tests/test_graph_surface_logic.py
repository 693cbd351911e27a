"""`Graph` (graph_gb300/graph.py) host logic on the CPU: a stand-in engine
records what the surface passes down, so the config mapping and merges, the
staging of arrays until render(), the onSimulation* callbacks and destroy()
are checked without a GPU (the engine itself is checked bit for bit against
the oracle by the GPU tests)."""
import math
import types

import numpy as np
import pytest

from graph_gb300 import _abi, graph


class StandInEngine:
    """A simulation of `ticks_to_end` ticks: start(alpha) runs it, each tick
    lowers alpha, and it ends when the ticks are used up."""

    ticks_to_end = 5

    def __init__(self, cfg):
        self.cfgs = [cfg]
        self.calls = []
        self.running = False
        self.paused = False
        self.alpha = 0.0
        self.ticks = 0

    def _log(self, name, *args):
        self.calls.append((name,) + args)

    def set_config(self, cfg):
        self.cfgs.append(cfg)

    def set_point_positions(self, a):
        self._log("positions", np.array(a, copy=True))

    def set_point_positions_ex(self, a, dont_rescale):
        self.dont_rescale = dont_rescale
        self._log("positions", np.array(a, copy=True))

    def set_links(self, a):
        self._log("links", np.array(a, copy=True))

    def set_link_strength(self, a):
        self._log("strength", a)

    def set_point_sizes(self, a):
        self._log("sizes", a)

    def set_point_clusters(self, a):
        self._log("clusters", a)

    def set_cluster_positions(self, a):
        self._log("cluster_positions", a)

    def set_point_cluster_strength(self, a):
        self._log("cluster_strength", a)

    def set_pinned_points(self, a):
        self._log("pinned", a)

    def render(self, alpha=None):
        self._log("render", alpha)

    def state(self):
        return types.SimpleNamespace(is_simulation_running=self.running and not self.paused, alpha=self.alpha,
                                     progress=self.ticks / self.ticks_to_end)

    def start(self, alpha):
        self.running, self.paused, self.alpha, self.ticks = True, False, alpha, 0

    def stop(self):
        self.running, self.alpha, self.ticks = False, 0.0, 0

    def pause(self):
        self.paused = True

    def unpause(self):
        self.paused = False

    def _tick(self):
        if not (self.running and not self.paused):
            return 0
        self.ticks += 1
        self.alpha *= 0.5
        if self.ticks >= self.ticks_to_end:
            self.running = False
        return 1

    def step(self, n):
        for _ in range(n):
            self._tick()

    def run(self, n):
        return sum(self._tick() for _ in range(n))

    def frame(self, n):
        return self.run(n)

    def get_point_positions(self):
        return getattr(self, "current", np.zeros(4, np.float32))

    def set_pointer(self, x, y, right):
        self._log("pointer", x, y, right)

    def set_drag(self, index):
        self._log("drag", index)

    def close(self):
        self._log("close")


@pytest.fixture
def make(monkeypatch):
    monkeypatch.setattr(graph, "Engine", StandInEngine)

    def build(config=None):
        events = []
        cfg = dict(config or {})
        for name in graph._CALLBACKS:
            cfg.setdefault(name, (lambda n: (lambda *a: events.append(n)))(name))
        g = graph.Graph(cfg)
        g.events = events
        return g
    return build


def test_config_maps_camel_case_and_ignores_visual_keys(make):
    g = make({"spaceSize": 2048, "simulationGravity": 0.5, "pointColor": "#fff", "enableDrag": True,
              "simulationCollisionRadius": None, "randomSeed": 7})
    cfg = g.engine.cfgs[0]
    assert cfg.space_size == 2048 and cfg.simulation_gravity == 0.5
    assert cfg.enable_drag == 1
    assert math.isnan(cfg.simulation_collision_radius)
    assert cfg.has_random_seed == 1 and cfg.random_seed == _abi.seed_to_u64(7)


def test_set_config_keeps_the_seed_and_partial_merges(make):
    g = make({"simulationGravity": 0.5, "simulationFriction": 0.7, "randomSeed": 3})
    g.setConfigPartial({"simulationFriction": 0.9, "randomSeed": 99})
    assert g.config["simulationGravity"] == 0.5 and g.config["simulationFriction"] == 0.9
    assert g.config["randomSeed"] == 3                       # the seed is fixed at creation
    g.setConfigPartial({"simulationGravity": None})          # undefined resets to the default
    assert "simulationGravity" not in g.config
    assert g.engine.cfgs[-1].simulation_gravity == _abi.DEFAULTS["simulation_gravity"]
    g.setConfig({"simulationFriction": 0.8})                 # a whole config replaces the others
    assert set(k for k in g.config if not k.startswith("on")) == {"simulationFriction", "randomSeed"}


def test_arrays_are_staged_by_reference_until_render(make):
    g = make()
    pos = np.zeros(4, np.float32)
    g.setPointPositions(pos)
    g.setLinks(np.array([0, 1], np.float32))
    pos[0] = 42.0                                            # changed after the setter, before render
    assert [c[0] for c in g.engine.calls] == []
    g.render(0.5)
    names = [c[0] for c in g.engine.calls]
    assert names == ["positions", "links", "render"]
    assert g.engine.calls[0][1][0] == 42.0
    assert g.engine.calls[-1] == ("render", 0.5)
    g.render()
    assert [c[0] for c in g.engine.calls][3:] == ["render"]  # nothing staged twice


def test_callbacks_follow_the_simulation_state(make):
    g = make()
    g.start(1.0)
    g.pause()
    g.pause()                                                # already paused: no second event
    g.unpause()
    n = g.run(100)
    assert n == StandInEngine.ticks_to_end
    assert g.events[:3] == ["onSimulationStart", "onSimulationPause", "onSimulationUnpause"]
    assert g.events[3:-1] == ["onSimulationTick"] * n
    assert g.events[-1] == "onSimulationEnd"
    assert not g.isSimulationRunning and g.progress == 1.0


def test_step_reports_every_tick_and_stop_ends(make):
    g = make()
    g.start(1.0)
    g.step(3)
    assert g.events == ["onSimulationStart"] + ["onSimulationTick"] * 3
    g.stop()
    assert g.events[-1] == "onSimulationEnd"
    g.stop()                                                 # nothing left to end
    assert g.events.count("onSimulationEnd") == 1


def test_drag_and_pointer_pass_through(make):
    g = make({"enableDrag": True})
    g.setPointer(10.0, 20.0, True)
    g.startDrag(3)
    g.endDrag()
    assert g.engine.calls == [("pointer", 10.0, 20.0, True), ("drag", 3), ("drag", None)]
    assert g.events == ["onDragStart", "onDragEnd"]


def test_everything_is_a_no_op_after_destroy(make):
    g = make()
    eng = g.engine
    g.destroy()
    g.destroy()
    assert eng.calls == [("close",)]
    g.setPointPositions(np.zeros(2, np.float32))
    g.render()
    g.start()
    g.step(2)
    assert g.run(5) == 0 and g.frame(2) == 0
    assert g.getPointPositions().size == 0
    assert not g.isSimulationRunning and g.progress == 0.0
    assert eng.calls == [("close",)]


def test_rescale_flags_and_write_back(make):
    # rescalePositions true: the engine rescales at render and the caller's
    # Float32Array receives the rescaled live positions (the reference writes it
    # in place, Points/index.ts:3211-3216); absent points stay as they were
    g = make({"rescalePositions": True})
    assert g.engine.cfgs[0].rescale_positions == 1
    pos = np.array([1.0, 2.0, np.nan, 5.0, 3.0, 4.0], np.float32)
    g.setPointPositions(pos)
    g.engine.current = np.array([10.0, 20.0, np.nan, np.nan, 30.0, 40.0], np.float32)
    g.render()
    assert g.engine.dont_rescale is False
    assert pos[0] == 10.0 and pos[5] == 40.0 and np.isnan(pos[2]) and pos[3] == 5.0
    # dontRescale skips it once (src/index.ts:553); nothing is written back
    pos2 = np.array([1.0, 2.0, 3.0, 4.0], np.float32)
    g.setPointPositions(pos2, True)
    g.engine.current = np.array([9.0, 9.0, 9.0, 9.0], np.float32)
    g.render()
    assert g.engine.dont_rescale is True and pos2[0] == 1.0
    # undefined rescales when the simulation is off (Points/index.ts:396-398)
    assert make({"enableSimulation": False})._rescales(False)
    assert not make({})._rescales(False)
    assert not make({"rescalePositions": False, "enableSimulation": False})._rescales(False)
    assert make({}).engine.cfgs[0].rescale_positions == -1

"""`Graph` — the reference's simulation surface over the GB300 engine.

Mirrors cosmos.gl's `Graph` (src/index.ts) for the parts that drive the force
simulation: setPointPositions / setLinks / setLinkStrength / setPointSizes /
setPinnedPoints / setPointClusters / setClusterPositions /
setPointClusterStrength / render / start / stop / pause / unpause / step /
getPointPositions / getClusterPositions / progress / isSimulationRunning / setConfig /
setConfigPartial / destroy, and the onSimulation* callbacks.  Rendering,
zoom, hover and picking stay in the browser and are not part of this class.

As in the reference, setters stage their array BY REFERENCE and the data is
read when `render()` runs (src/index.ts:548-574, GraphData/index.ts:123-127);
every method is a silent no-op after `destroy()`.
"""
import math

import numpy as np

from . import _abi
from .engine import Engine

ALPHA_MIN = 0.001

_CALLBACKS = ("onSimulationStart", "onSimulationTick", "onSimulationEnd", "onSimulationPause",
              "onSimulationUnpause", "onDragStart", "onDragEnd")


def _to_fields(config):
    fields = {}
    for k, v in (config or {}).items():
        if k in _CALLBACKS:
            continue
        f = _abi.CAMEL_TO_FIELD.get(k)
        if f is None:
            continue   # visual keys of the reference are accepted and ignored here
        if f == "simulation_collision_radius" and v is None:
            v = math.nan
        if f in ("enable_simulation", "enable_right_click_repulsion", "enable_drag"):
            v = 1 if v else 0
        if f == "rescale_positions":
            v = -1 if v is None else (1 if v else 0)
        fields[f] = v
    return fields


class Graph:
    def __init__(self, config=None, device=0):
        config = dict(config or {})
        self._callbacks = {k: config.get(k) for k in _CALLBACKS}
        self._config = dict(config)
        fields = _to_fields(config)
        # randomSeed seeds the reference's stream with String(randomSeed) (src/index.ts:452)
        cfg = _abi.make_config(device=device, **fields)
        self._engine = Engine(cfg)
        self._destroyed = False
        self._staged = {}

    # --- config (src/index.ts:500-530) -------------------------------------
    def _apply(self, merged):
        self._callbacks = {k: merged.get(k) for k in _CALLBACKS}
        fields = _to_fields(merged)
        fields.pop("random_seed", None)
        cfg = _abi.make_config(**fields)
        self._engine.set_config(cfg)
        self._config = merged

    def setConfig(self, config):
        if self._destroyed:
            return
        merged = dict(config or {})
        if "randomSeed" in self._config:
            merged["randomSeed"] = self._config["randomSeed"]
        self._apply(merged)

    def setConfigPartial(self, config):
        if self._destroyed:
            return
        merged = dict(self._config)
        for k, v in (config or {}).items():
            if k == "randomSeed":
                continue
            if v is None:
                merged.pop(k, None)   # explicit undefined resets to the default (config.ts:866-881)
            else:
                merged[k] = v
        self._apply(merged)

    @property
    def config(self):
        return dict(self._config)

    # --- data (staged by reference, read at render) -------------------------
    def setPointPositions(self, pointPositions, dontRescale=None):
        """Stage positions; dontRescale skips the next render's rescale (src/index.ts:548-553)."""
        if self._destroyed:
            return
        self._staged["positions"] = pointPositions
        self._staged["dont_rescale"] = bool(dontRescale)

    def setLinks(self, links):
        if self._destroyed:
            return
        self._staged["links"] = links

    def setLinkStrength(self, linkStrength):
        if self._destroyed:
            return
        self._staged["strength"] = linkStrength

    def setPointSizes(self, pointSizes):
        if self._destroyed:
            return
        self._staged["sizes"] = pointSizes

    def setPointClusters(self, pointClusters):
        """Cluster index per point; None (the reference's `undefined`) = no cluster (src/index.ts:854-859)."""
        if self._destroyed:
            return
        self._staged["clusters"] = pointClusters

    def setClusterPositions(self, clusterPositions):
        """x, y per cluster; None = centre of mass (src/index.ts:871-876)."""
        if self._destroyed:
            return
        self._staged["cluster_positions"] = clusterPositions

    def setPointClusterStrength(self, clusterStrength):
        """Per-point coefficient of the cluster pull (src/index.ts:888-893)."""
        if self._destroyed:
            return
        self._staged["cluster_strength"] = clusterStrength

    def setPinnedPoints(self, pinnedIndices):
        if self._destroyed:
            return
        idx = None if pinnedIndices is None or len(pinnedIndices) == 0 else pinnedIndices
        self._engine.set_pinned_points(idx)

    def render(self, simulationAlpha=None, transitionDuration=None):
        if self._destroyed:
            return
        s = self._staged
        rescaled = None
        if "positions" in s:
            positions = s.pop("positions")
            dont = s.pop("dont_rescale", False)
            self._engine.set_point_positions_ex(positions, dont)
            if self._rescales(dont):
                rescaled = positions
        if "links" in s:
            self._engine.set_links(s.pop("links"))
        if "strength" in s:
            self._engine.set_link_strength(s.pop("strength"))
        if "sizes" in s:
            self._engine.set_point_sizes(s.pop("sizes"))
        if "clusters" in s:
            self._engine.set_point_clusters(s.pop("clusters"))
        if "cluster_positions" in s:
            self._engine.set_cluster_positions(s.pop("cluster_positions"))
        if "cluster_strength" in s:
            self._engine.set_point_cluster_strength(s.pop("cluster_strength"))
        self._engine.render(simulationAlpha)
        if isinstance(rescaled, np.ndarray) and rescaled.dtype == np.float32 and rescaled.flags.writeable:
            # the reference rescales the caller's Float32Array in place
            # (Points/index.ts:3211-3216): copy the rescaled live positions back
            now = self._engine.get_point_positions()
            if now.size == rescaled.size:
                flat = rescaled.reshape(-1)
                live = ~(np.isnan(flat[0::2]) | np.isnan(flat[1::2]))
                flat[0::2][live] = now[0::2][live]
                flat[1::2][live] = now[1::2][live]

    def _rescales(self, dont_rescale):
        # Points.updatePositions (Points/index.ts:396-402)
        r = self._config.get("rescalePositions")
        if r is None and not self._config.get("enableSimulation", True):
            r = True
        return bool(r) and not dont_rescale

    # --- control (src/index.ts:1457-1540) ------------------------------------
    def _cb(self, name, *args):
        fn = self._callbacks.get(name)
        if fn:
            fn(*args)

    def start(self, alpha=1.0):
        if self._destroyed:
            return
        before = self._engine.state()
        self._engine.start(alpha)
        after = self._engine.state()
        if after.is_simulation_running and not before.is_simulation_running:
            self._cb("onSimulationStart")

    def stop(self):
        if self._destroyed:
            return
        s = self._engine.state()
        was_active = s.is_simulation_running or s.alpha > 0 or s.progress > 0
        self._engine.stop()
        if was_active:
            self._cb("onSimulationEnd")

    def pause(self):
        if self._destroyed:
            return
        if not self._engine.state().is_simulation_running:
            return
        self._engine.pause()
        self._cb("onSimulationPause")

    def unpause(self):
        if self._destroyed:
            return
        if self._engine.state().is_simulation_running:
            return
        self._engine.unpause()
        if self._engine.state().is_simulation_running:
            self._cb("onSimulationUnpause")

    def step(self, ticks=1):
        """Graph.step(); `ticks` > 1 runs that many steps in one call."""
        if self._destroyed:
            return
        if self._callbacks.get("onSimulationTick"):
            for _ in range(int(ticks)):
                self._engine.step(1)
                self._cb("onSimulationTick", self._engine.state().alpha, None, None)
        else:
            self._engine.step(int(ticks))

    def run(self, maxTicks):
        """The animation-frame loop: tick while running, end once alpha < ALPHA_MIN."""
        if self._destroyed:
            return 0
        was_running = self._engine.state().is_simulation_running
        if self._callbacks.get("onSimulationTick"):
            n = 0
            while n < maxTicks:
                done = self._engine.run(1)
                if done == 0:
                    break
                n += 1
                self._cb("onSimulationTick", self._engine.state().alpha, None, None)
        else:
            n = self._engine.run(int(maxTicks))
        if was_running and not self._engine.state().is_simulation_running:
            self._cb("onSimulationEnd")
        return n

    # --- read-back -------------------------------------------------------------
    def getPointPositions(self):
        """Positions as float32 [x0, y0, x1, y1, ...]; absent points read NaN."""
        if self._destroyed:
            return np.zeros(0, dtype=np.float32)
        return self._engine.get_point_positions()

    # --- interaction (the reference takes these from DOM pointer events) ----
    def setPointer(self, x, y, rightButton=False):
        """Pointer in simulation space and the right button (Store.mousePosition, isRightClickMouse)."""
        if self._destroyed:
            return
        self._engine.set_pointer(x, y, rightButton)

    def startDrag(self, index):
        """Drag.start on the hovered point `index` (Drag/index.ts:22-28); needs enableDrag."""
        if self._destroyed:
            return
        self._engine.set_drag(index)
        self._cb("onDragStart")

    def endDrag(self):
        if self._destroyed:
            return
        self._engine.set_drag(None)
        self._cb("onDragEnd")

    def frame(self, frames=1):
        """Run `frames` animation frames' simulation work; returns the ticks run."""
        if self._destroyed:
            return 0
        running = self._engine.state().is_simulation_running
        done = self._engine.frame(frames)
        if running and not self._engine.state().is_simulation_running:
            self._cb("onSimulationEnd")
        return done

    def getPositionTexture(self):
        """The renderer's points texture (Points/position-utils.ts:9-27): float32 (T*T, 4) of
        (x, y, index, 0); the engine writes it in the layout the draw passes read."""
        if self._destroyed:
            return np.zeros((0, 4), dtype=np.float32)
        return self._engine.get_position_texture()

    def getClusterPositions(self):
        """Centre of mass of each cluster as float64 [x0, y0, x1, y1, ...] (src/index.ts:1135-1139)."""
        if self._destroyed:
            return np.zeros(0, dtype=np.float64)
        return self._engine.get_cluster_positions()

    @property
    def progress(self):
        return 0.0 if self._destroyed else self._engine.state().progress

    @property
    def isSimulationRunning(self):
        return False if self._destroyed else bool(self._engine.state().is_simulation_running)

    @property
    def engine(self):
        return self._engine

    def destroy(self):
        if self._destroyed:
            return
        self._destroyed = True
        self._engine.close()

"""Typed numpy-facing wrapper over an engine-style C API (prefix + handle).

Shared by the product's ctypes binding (graph_gb300.engine.Engine) and the
parity oracle's binding, so that both are driven by identical calls.
"""
import ctypes as C
import math

import numpy as np

from . import _abi


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class StatusError(RuntimeError):
    def __init__(self, fn, status, text=""):
        self.status = status
        super().__init__("%s failed: %s %s" % (fn, _abi.STATUS_NAMES.get(status, status), text))


class EngineCalls:
    """Subclasses set self._lib, self._prefix, self._h and implement _err_text()."""

    _lib = None
    _prefix = ""
    _h = None
    last_status = 0

    def _fn(self, name):
        return getattr(self._lib, "%s_%s" % (self._prefix, name))

    def _err_text(self):
        return ""

    def _check(self, name, st):
        self.last_status = st
        if st not in (_abi.CGL_OK, _abi.CGL_WARNING):
            raise StatusError("%s_%s" % (self._prefix, name), st, self._err_text())
        return st

    def _call(self, name, *args):
        return self._check(name, self._fn(name)(self._h, *args))

    # --- simulation surface -------------------------------------------------
    def set_point_positions(self, xy):
        a = _f32(xy)
        return self._call("set_point_positions", _fptr(a), a.size)

    def set_point_positions_ex(self, xy, dont_rescale):
        a = _f32(xy)
        return self._call("set_point_positions_ex", _fptr(a), a.size, 1 if dont_rescale else 0)

    def set_links(self, st):
        a = _f32(st)
        return self._call("set_links", _fptr(a), a.size)

    def set_link_strength(self, s):
        if s is None:
            return self._call("set_link_strength", None, 0)
        a = _f32(s)
        return self._call("set_link_strength", _fptr(a), a.size)

    def set_point_sizes(self, s):
        if s is None:
            return self._call("set_point_sizes", None, 0)
        a = _f32(s)
        return self._call("set_point_sizes", _fptr(a), a.size)

    def set_pinned_points(self, idx):
        if idx is None or len(idx) == 0:
            return self._call("set_pinned_points", None, 0)
        a = np.ascontiguousarray(np.asarray(idx, dtype=np.float64))
        return self._call("set_pinned_points", a.ctypes.data_as(C.POINTER(C.c_double)), a.size)

    def set_point_clusters(self, clusters):
        """One value per point; None or NaN = no cluster (the reference's `undefined`)."""
        if clusters is None:
            return self._call("set_point_clusters", None, 0)
        a = _f32([math.nan if v is None else v for v in clusters]
                 if isinstance(clusters, (list, tuple)) else clusters)
        return self._call("set_point_clusters", _fptr(a), a.size)

    def set_cluster_positions(self, xy):
        """x, y per cluster; None or NaN = centre of mass.  None clears them."""
        if xy is None:
            return self._call("set_cluster_positions", None, 0)
        a = _f32([math.nan if v is None else v for v in xy] if isinstance(xy, (list, tuple)) else xy)
        if a.size == 0:
            a = np.zeros(1, dtype=np.float32)   # a non-null pointer: `[]` counts as set
            return self._call("set_cluster_positions", _fptr(a), 0)
        return self._call("set_cluster_positions", _fptr(a), a.size)

    def set_point_cluster_strength(self, s):
        if s is None:
            return self._call("set_point_cluster_strength", None, 0)
        a = _f32(s)
        return self._call("set_point_cluster_strength", _fptr(a), a.size)

    def get_cluster_positions(self):
        n = C.c_uint64(0)
        self._call("get_cluster_positions", None, 0, C.byref(n))
        out = np.empty(n.value, dtype=np.float64)
        if n.value:
            self._call("get_cluster_positions", out.ctypes.data_as(C.POINTER(C.c_double)), out.size, C.byref(n))
        return out

    def render(self, alpha=None):
        return self._call("render", math.nan if alpha is None else float(alpha))

    def start(self, alpha=1.0):
        return self._call("start", float(alpha))

    def stop(self):
        return self._call("stop")

    def pause(self):
        return self._call("pause")

    def unpause(self):
        return self._call("unpause")

    def step(self, ticks=1):
        return self._call("step", int(ticks))

    def set_pointer(self, x, y, right_button=False):
        return self._call("set_pointer", float(x), float(y), 1 if right_button else 0)

    def set_drag(self, index):
        return self._call("set_drag", -1 if index is None else int(index))

    def frame(self, frames=1):
        done = C.c_uint32(0)
        self._call("frame", int(frames), C.byref(done))
        return done.value

    def run(self, max_ticks):
        done = C.c_uint32(0)
        self._call("run", int(max_ticks), C.byref(done))
        return done.value

    def state(self):
        s = _abi.State()
        self._call("get_state", C.byref(s))
        return s

    def layout(self):
        s = _abi.Layout()
        self._call("get_layout", C.byref(s))
        return s

    def get_point_positions(self):
        n = self.layout().points_number
        out = np.empty(2 * n, dtype=np.float32)
        self._call("get_point_positions", _fptr(out), out.size)
        return out

    def set_config(self, cfg):
        return self._call("set_config", C.byref(cfg))

    # --- test hooks ---------------------------------------------------------
    def cells(self, level):
        lay = self.layout()
        g = 4 << level
        out = np.empty(4 * g * g, dtype=np.float32)
        self._call("debug_get_cells", int(level), _fptr(out), out.size)
        return out.reshape(g, g, 4)

    def slots(self):
        lay = self.layout()
        g = lay.finest_grid
        out = np.empty(8 * g * g, dtype=np.int32)
        self._call("debug_get_slots", out.ctypes.data_as(C.POINTER(C.c_int32)), out.size)
        return out.reshape(g, g, 8)

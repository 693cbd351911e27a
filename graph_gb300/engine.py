"""Typed binding of the engine's C ABI (include/cgl.h) over ctypes.

`load_library()` loads graph_gb300/libcgl_gb300.so (building it with nvcc if
it is missing and nvcc is available).  There is no CPU fallback: if the
library cannot be loaded, or no CUDA device is usable, engine creation raises.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from ._calls import EngineCalls, StatusError

_LIB = None
_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcgl_gb300.so")


def load_library(build_if_missing: bool = True):
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError("graph_gb300: %s is missing (run graph_gb300/build.py)" % LIB_PATH)
        from . import build
        build.build()
    lib = C.CDLL(LIB_PATH)
    E = C.c_void_p
    lib.cgl_config_defaults.argtypes = [C.POINTER(_abi.Config)]
    lib.cgl_config_defaults.restype = None
    lib.cgl_create.argtypes = [C.POINTER(_abi.Config), C.POINTER(C.c_void_p)]
    lib.cgl_create.restype = C.c_int
    lib.cgl_destroy.argtypes = [E]
    lib.cgl_destroy.restype = C.c_int
    lib.cgl_last_error.argtypes = [E]
    lib.cgl_last_error.restype = C.c_char_p
    lib.cgl_get_config.argtypes = [E, C.POINTER(_abi.Config)]
    lib.cgl_get_config.restype = C.c_int
    lib.cgl_set_stream.argtypes = [E, C.c_void_p]
    lib.cgl_set_stream.restype = C.c_int
    lib.cgl_synchronize.argtypes = [E]
    lib.cgl_synchronize.restype = C.c_int
    lib.cgl_profile_stages.argtypes = [E, C.c_uint32, C.POINTER(C.c_double)]
    lib.cgl_profile_stages.restype = C.c_int
    for name in ("cgl_get_position_texture", "cgl_enqueue_position_texture"):
        getattr(lib, name).argtypes = [E, C.c_void_p, C.c_uint64]
        getattr(lib, name).restype = C.c_int
    lib.cgl_levels_noalloc.argtypes = [C.c_void_p, C.c_uint64, C.c_double, C.c_void_p, C.c_uint64, C.c_void_p,
                                       C.c_char_p, C.c_size_t]
    lib.cgl_levels_noalloc.restype = C.c_int
    lib.cgl_random_draws.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(C.c_double)]
    lib.cgl_random_draws.restype = C.c_int
    lib.cgl_check_wait_limit.argtypes = [C.c_int32, C.POINTER(C.c_uint32)]
    lib.cgl_check_wait_limit.restype = C.c_int
    lib.cgl_enqueue_point_positions.argtypes = [E, C.POINTER(C.c_float), C.c_uint64]
    lib.cgl_enqueue_point_positions.restype = C.c_int
    lib.cgl_debug_set_leading_hubs.argtypes = [E, C.c_int32, C.c_int32]
    lib.cgl_debug_set_leading_hubs.restype = C.c_int
    _abi.declare(lib, "cgl")
    _LIB = lib
    return lib


class Engine(EngineCalls):
    """One engine handle: one CUDA stream on one device."""

    def __init__(self, cfg=None, **fields):
        self._lib = load_library()
        self._prefix = "cgl"
        if cfg is None:
            cfg = _abi.make_config(**fields)
        h = C.c_void_p()
        st = self._lib.cgl_create(C.byref(cfg), C.byref(h))
        if st != _abi.CGL_OK:
            raise StatusError("cgl_create", st, "(no usable CUDA device?)")
        self._h = h

    def _err_text(self):
        if not self._h:
            return ""
        t = self._lib.cgl_last_error(self._h)
        return t.decode() if t else ""

    def last_error(self):
        return self._err_text()

    def close(self):
        if self._h:
            self._lib.cgl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def config(self):
        c = _abi.Config()
        self._call("get_config", C.byref(c))
        return c

    def set_stream(self, stream_ptr):
        return self._call("set_stream", C.c_void_p(stream_ptr) if stream_ptr else None)

    def synchronize(self):
        return self._call("synchronize")

    def set_leading_hubs(self, max_in, max_out=None):
        """Test hook: the first max_in incoming and max_out (default max_in) outgoing hub lists
        lead whatever their lengths (0: none, -1: the engine's rule)."""
        return self._call("debug_set_leading_hubs", int(max_in), int(max_in if max_out is None else max_out))

    def profile_stages(self, ticks):
        out = (C.c_double * _abi.NUM_STAGE_TIMES)()
        self._call("profile_stages", int(ticks), out)
        return dict(zip(_abi.STAGE_TIME_NAMES, list(out)))

    def get_position_texture(self):
        """The renderer's points texture: float32 [T*T, 4] of (x, y, index, 0)."""
        t = self.layout().points_texture_size
        out = np.empty((t * t, 4), dtype=np.float32)
        self._call("get_position_texture", C.c_void_p(out.ctypes.data), out.size)
        return out

    def get_position_texture_into(self, ptr, capacity_floats):
        """Write the texture to `ptr` (host, pinned host or device memory) and wait."""
        return self._call("get_position_texture", C.c_void_p(ptr), int(capacity_floats))

    def enqueue_position_texture(self, ptr, capacity_floats):
        """Queue the texture write to device or pinned host memory at `ptr` (done by the next synchronize)."""
        return self._call("enqueue_position_texture", C.c_void_p(ptr), int(capacity_floats))

    def enqueue_point_positions_into(self, out):
        """Queue the positions' read-back into a pinned host (or device) float32 buffer beside the
        next ticks; returns once the previously queued read-back has landed."""
        n = self.layout().points_number
        assert out.dtype == np.float32 and out.size >= 2 * n
        return self._call("enqueue_point_positions", out.ctypes.data_as(C.POINTER(C.c_float)), out.size)

    def get_point_positions_into(self, out):
        """Read positions into a caller-owned float32 buffer (e.g. pinned host memory)."""
        n = self.layout().points_number
        assert out.dtype == np.float32 and out.size >= 2 * n
        return self._call("get_point_positions", out.ctypes.data_as(C.POINTER(C.c_float)), out.size)

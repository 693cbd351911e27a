"""Parity oracle for the GB300 force-layout engine — TEST INFRASTRUCTURE.

A CPU restatement (oracle/oracle.cpp) of cosmos.gl's per-tick simulation,
driven through the same call surface as the engine.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and only as
the checker or the timed CPU baseline.  Parity is unpinned by the reference
(it has no tests or golden vectors and cannot execute here); see the header of
oracle.cpp.
"""
import ctypes as C
import os

import numpy as np

from graph_gb300 import _abi
from graph_gb300._calls import EngineCalls

from . import build as _build

_LIB = None


def load():
    global _LIB
    if _LIB is None:
        path = _build.build()
        lib = C.CDLL(path)
        lib.orc_create.argtypes = [C.POINTER(_abi.Config)]
        lib.orc_create.restype = C.c_void_p
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_destroy.restype = None
        lib.orc_set_sum_mode.argtypes = [C.c_void_p, C.c_int]
        lib.orc_set_sum_mode.restype = None
        _abi.declare(lib, "orc")
        lib.orc_lowbias32.argtypes = [C.c_uint32]
        lib.orc_lowbias32.restype = C.c_uint32
        lib.orc_peel_hash.argtypes = [C.c_uint32, C.c_uint32]
        lib.orc_peel_hash.restype = C.c_float
        lib.orc_splitmix_draw.argtypes = [C.c_uint64, C.c_uint64]
        lib.orc_splitmix_draw.restype = C.c_uint64
        lib.orc_seedrandom.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(C.c_double)]
        lib.orc_seedrandom.restype = None
        lib.orc_sincos.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_sincos.restype = None
        lib.orc_cell_index.argtypes = [C.c_float, C.c_float, C.c_int]
        lib.orc_cell_index.restype = C.c_int
        lib.orc_manybody_velocity.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        lib.orc_manybody_velocity.restype = C.c_int
        lib.orc_debug_get_csr.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 5
        lib.orc_debug_get_csr.restype = C.c_int
        lib.orc_debug_get_jitter.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_uint64]
        lib.orc_debug_get_jitter.restype = C.c_int
        _LIB = lib
    return _LIB


class OracleEngine(EngineCalls):
    """Same methods as graph_gb300.engine.Engine, computed on the CPU."""

    def __init__(self, cfg=None, sum_mode=0, **fields):
        self._lib = load()
        self._prefix = "orc"
        if cfg is None:
            cfg = _abi.make_config(**fields)
        self._h = C.c_void_p(self._lib.orc_create(C.byref(cfg)))
        self._lib.orc_set_sum_mode(self._h, int(sum_mode))

    def close(self):
        if self._h:
            self._lib.orc_destroy(self._h)
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

    def manybody_velocity(self, precision=0):
        n = self.layout().points_number
        out = np.zeros(2 * n, dtype=np.float64)
        st = self._lib.orc_manybody_velocity(self._h, int(precision), out.ctypes.data_as(C.POINTER(C.c_double)))
        self._check("manybody_velocity", st)
        return out

    def csr(self, direction):
        lay = self.layout()
        n = lay.points_number
        m = lay.link_entries_in
        rowptr = np.zeros(n + 1, dtype=np.uint32)
        col = np.zeros(m, dtype=np.uint32)
        rnd = np.zeros(m, dtype=np.float32)
        bias = np.zeros(m, dtype=np.float32)
        strength = np.zeros(m, dtype=np.float32)
        self._lib.orc_debug_get_csr(self._h, int(direction), rowptr.ctypes.data, col.ctypes.data,
                                    rnd.ctypes.data, bias.ctypes.data, strength.ctypes.data)
        return dict(rowptr=rowptr, col=col, rnd=rnd, bias=bias, strength=strength)

    def jitter(self):
        n = self.layout().points_number
        out = np.zeros(2 * n, dtype=np.float32)
        self._lib.orc_debug_get_jitter(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), out.size)
        return out


def lowbias32(h):
    return load().orc_lowbias32(h)


def peel_hash(index, seed_bits):
    return load().orc_peel_hash(index, seed_bits)


def splitmix_draw(seed, k):
    return load().orc_splitmix_draw(seed, k)


def seedrandom(seed_text, n):
    """The oracle's restatement of seedrandom@3.0.5: its first n values for seed_text."""
    out = np.zeros(n, dtype=np.float64)
    load().orc_seedrandom(str(seed_text).encode("utf-8"), n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def sincos(a):
    s = C.c_float()
    c = C.c_float()
    load().orc_sincos(a, C.byref(s), C.byref(c))
    return s.value, c.value


def cell_index(p, cs, g):
    return load().orc_cell_index(p, cs, g)

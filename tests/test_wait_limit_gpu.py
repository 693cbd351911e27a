"""The one-pass cell scans' bounded wait (device_util.cuh, scan_look_back).

A scan block waits for the status words of the chunks before its own.  Every
such chunk belongs to a block that has started, so the wait ends; it still
carries a poll limit, after which the block raises its error bit in a
host-mapped word and returns, and the engine reports CGL_CUDA_ERROR at its next
synchronisation.  Here the wait runs against a status word that nothing sets:
it must give up by itself, raise the bit and leave the context usable.
"""
import ctypes as C
import time

import numpy as np
import pytest

from graph_gb300 import _abi, generators

pytestmark = pytest.mark.gpu


def test_wait_gives_up_and_reports():
    from graph_gb300.engine import Engine, load_library
    lib = load_library()
    bits = C.c_uint32(0)
    t0 = time.perf_counter()
    assert lib.cgl_check_wait_limit(0, C.byref(bits)) == _abi.CGL_OK
    took = time.perf_counter() - t0
    assert bits.value == _abi.CGL_ERROR_SCAN
    assert took < 30.0, took
    # the context still runs an engine afterwards
    e = Engine(random_seed=3)
    e.set_point_positions(generators.uniform_positions(2000, 0, 4096, 3))
    e.render()
    e.start(1.0)
    e.step(3)
    e.synchronize()
    assert np.isfinite(e.get_point_positions()).all()
    e.close()


"""CPU tests of the C ABI library: it builds, loads, exports every declared
symbol, and its defaults match the reference.  No compute calls (no GPU here)."""
import ctypes as C
import math
import os
import re

import pytest

from graph_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cgl.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cgl_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_simulation_surface():
    names = declared_functions()
    for fn in ["cgl_create", "cgl_destroy", "cgl_set_config", "cgl_set_point_positions", "cgl_set_links",
               "cgl_set_link_strength", "cgl_set_point_sizes", "cgl_set_pinned_points", "cgl_render",
               "cgl_start", "cgl_stop", "cgl_pause", "cgl_unpause", "cgl_step", "cgl_run",
               "cgl_get_point_positions", "cgl_get_state", "cgl_last_error"]:
        assert fn in names


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [fn for fn in declared_functions() if not hasattr(engine_lib, fn)]
    assert not missing, missing


def test_config_defaults_match_reference(engine_lib):
    c = _abi.Config()
    engine_lib.cgl_config_defaults(C.byref(c))
    got = _abi.config_to_dict(c)
    for k, v in _abi.DEFAULTS.items():
        if isinstance(v, float) and math.isnan(v):
            assert math.isnan(got[k]), k
        elif k == "simulation_link_dist_random_variation_range":
            assert tuple(got[k]) == tuple(v)
        else:
            assert got[k] == v, k


def test_struct_sizes_match_header():
    # natural C layout: doubles and uint64 aligned to 8
    assert C.sizeof(_abi.Config) == 216
    assert C.sizeof(_abi.State) == 56
    assert C.sizeof(_abi.Layout) == 104
    assert C.sizeof(_abi.BatchJob) == 64


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from graph_gb300.engine import Engine
    from graph_gb300._calls import StatusError
    with pytest.raises(StatusError):
        Engine(random_seed=1)


def test_seed_mapping():
    assert _abi.seed_to_u64(5) == 5
    assert _abi.seed_to_u64(-1) == (1 << 64) - 1
    assert _abi.seed_to_u64("abc") == _abi.seed_to_u64("abc") != _abi.seed_to_u64("abd")
    assert _abi.seed_to_u64(2.0) == 2


def test_layout_names_the_many_body_kernels():
    src = open(HEADER).read()
    for name, value in (("CGL_MANYBODY_ONE_POINT", 0), ("CGL_MANYBODY_SPLIT", 1), ("CGL_MANYBODY_TWO_POINTS", 2)):
        assert re.search(r"%s = %d" % (name, value), src)
    assert (_abi.MANYBODY_ONE_POINT, _abi.MANYBODY_SPLIT, _abi.MANYBODY_TWO_POINTS) == (0, 1, 2)
    assert [f for f, _ in _abi.Layout._fields_][-5:] == ["manybody_kernel", "manybody_tuned", "early_hubs",
                                                         "early_points", "leading_out_hubs"]


def test_create_rejects_an_unknown_manybody_kernel(engine_lib):
    # checked before any device call, so it runs without a GPU
    for bad in (-2, 3, 99):
        cfg = _abi.make_config(manybody_kernel=bad)
        h = C.c_void_p()
        assert engine_lib.cgl_create(C.byref(cfg), C.byref(h)) == _abi.CGL_INVALID_ARG

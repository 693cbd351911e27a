"""bench.py's byte models and stage filter (host code, no GPU)."""
import importlib.util
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(HERE, "..", "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def test_tick_bytes_model():
    b = _bench()
    # the 1M-point SBM: N = 1e6, E = 4,976,035 links, 512^2 finest cells
    assert b.tick_bytes(1_000_000, 4_976_035, 512 * 512) == 112_000_000 + 48 * 4_976_035 + 107 * 262_144
    assert b.tick_bytes(10, 20, 16, cc=4) == 112 * 10 + 48 * 20 + 107 * 16 + 144 * 10 + 128 * 4


def test_stages_without_work_are_left_out():
    b = _bench()
    timed = {"prepass": 0.0235, "center": 0.0021, "manybody": 0.37, "clusters": 0.0}
    assert b.ran_stages(timed, {"simulation_center": 0.0}) == {"prepass": 0.0235, "manybody": 0.37}
    assert b.ran_stages(timed, {"simulation_center": 0.1}) == {"prepass": 0.0235, "center": 0.0021,
                                                               "manybody": 0.37}


def test_stage_bytes_cover_every_timed_stage():
    b = _bench()
    from graph_gb300 import _abi
    for name in _abi.STAGE_TIME_NAMES:
        if name.startswith("collision") or name in ("prepass", "center", "scan", "scatter", "cells", "manybody",
                                                    "link_in", "link_out", "clusters"):
            assert b.stage_bytes(name, 10, 20, 16, 21) > 0


def test_reference_arm_is_recognised_before_imports():
    b = _bench()
    assert b._reference_arm(["--impl", "reference", "--gpus", "2"])
    assert b._reference_arm(["--steps", "3", "--impl=reference"])
    assert not b._reference_arm(["--impl", "gb300"])
    assert not b._reference_arm(["--gpus", "2"])


def test_rel_errors():
    b = _bench()
    ref = np.array([1.0, 0.0, 0.0, 2.0, 0.0, 0.0])
    v = np.array([1.1, 0.0, 0.0, 2.0, 0.5, 0.0])
    e = b.rel_errors(v, ref)
    assert e["points"] == 2 and abs(e["max_rel"] - 0.1) < 1e-12
    assert abs(e["rms_rel"] - math.sqrt((0.01 + 0.25) / 3 / (5 / 3))) < 1e-12


def test_issue_roofline_uses_the_ncu_instruction_count():
    b = _bench()
    ncu = {"file": "ncu_x.json", "state": "ticks 5-7", "kernels": {"manybody": {"inst_executed": 1.0e8,
                                                                                "dram_bytes": 2.0e7}}}
    r = b.issue_roofline("manybody", 0.5, ncu, 152, 2000.0, 29e6, 6000.0, "measured")
    assert r["bound"] == "issue" and r["unit"] == "warp-inst/s"
    assert abs(r["achieved"] - 2.0e11) < 1 and abs(r["peak"] - 4 * 152 * 2.0e9) < 1
    assert abs(r["frac"] - 2.0e11 / (4 * 152 * 2.0e9)) < 1e-12
    assert r["traffic"] == 2.0e7 and abs(r["hbm"]["achieved"] - 58.0) < 1e-9
    r = b.issue_roofline("manybody", 0.5, {}, 152, 2000.0, 29e6, 6000.0, "measured")
    assert r["achieved"] is None and r["frac"] is None

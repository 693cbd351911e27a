"""The full-run agreement measures (graph_gb300/agreement.py) on known cases."""
import math

import numpy as np

from graph_gb300 import agreement


def test_identical_layouts_agree_exactly():
    rng = np.random.default_rng(1)
    a = rng.uniform(0, 100, size=200)
    links = rng.integers(0, 100, size=300).astype(np.float32)
    f = agreement.agreement(a, a.copy(), links)
    assert f == dict(procrustes_rms=0.0, procrustes_rms_relative=0.0, edge_length_stress=0.0)


def test_rotation_and_translation_are_aligned_away():
    rng = np.random.default_rng(2)
    a = rng.uniform(0, 100, size=(500, 2))
    th = 0.7
    r = np.array([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]])
    b = a @ r.T + np.array([30.0, -12.0])
    rms, rel = agreement.procrustes_rms(a.reshape(-1), b.reshape(-1))
    assert rms < 1e-9 and rel < 1e-11
    links = rng.integers(0, 500, size=800)
    assert agreement.edge_length_stress(a.reshape(-1), b.reshape(-1), links) < 1e-12


def test_known_displacement_and_stress():
    # two points 2 apart; b stretches them to 4 apart about the same centre
    a = np.array([-1.0, 0.0, 1.0, 0.0])
    b = np.array([-2.0, 0.0, 2.0, 0.0])
    rms, rel = agreement.procrustes_rms(a, b)
    assert abs(rms - 1.0) < 1e-12 and abs(rel - 1.0) < 1e-12
    assert abs(agreement.edge_length_stress(a, b, [0, 1]) - 1.0) < 1e-12
    rms_s, _ = agreement.procrustes_rms(a, b, scale=True)
    assert rms_s < 1e-12


def test_absent_points_and_bad_links_are_left_out():
    a = np.array([0.0, 0.0, 1.0, 0.0, np.nan, np.nan, 0.0, 1.0])
    b = a.copy()
    b[4:6] = [50.0, 50.0]
    assert agreement.procrustes_rms(a, b) == (0.0, 0.0)
    assert agreement.edge_length_stress(a, b, [0, 1, 1, 2, 0, 3, -1, 2, 2.5, 1, 0, 9]) == 0.0

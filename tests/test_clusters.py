"""Clusters force (Clusters/index.ts, force-cluster.frag, calculate-centermass.vert).

CPU tests pin the oracle's cluster semantics on tiny inputs; GPU tests hold the
engine to bitwise equality with the oracle, with few clusters (block-level
sums), many clusters (warp-level sums straight to memory), custom positions,
strengths, unclustered / invalid indices, absent and pinned points.
"""
import math

import numpy as np
import pytest

from graph_gb300 import _abi, generators

from helpers import first_mismatch, make_pair, same_bits, scenario

CL = _abi.STAGE_CLUSTERS


def _oracle(fields, pos, clusters=None, cluster_positions=None, strength=None):
    from oracle import OracleEngine
    o = OracleEngine(**fields)
    o.set_point_positions(np.asarray(pos, dtype=np.float32))
    if clusters is not None:
        o.set_point_clusters(clusters)
    if cluster_positions is not None:
        o.set_cluster_positions(cluster_positions)
    if strength is not None:
        o.set_point_cluster_strength(strength)
    o.render()
    o.start(1.0)
    return o


def test_cluster_count_and_centroids():
    pos = [100.0, 200.0, 300.0, 400.0, 1000.0, 1000.0, 7.0, 9.0]
    o = _oracle(dict(random_seed=1, stage_mask=CL), pos, clusters=[0, 0, 3, None])
    c = o.get_cluster_positions()
    assert c.size == 8                     # clusterCount = max index + 1 = 4
    assert c[0] == 200.0 and c[1] == 300.0
    assert np.isnan(c[2]) and np.isnan(c[3])   # cluster 1 has no point: 0/0 as in the reference
    assert c[6] == 1000.0 and c[7] == 1000.0


def test_invalid_indices_are_unclustered():
    pos = [100.0, 200.0, 300.0, 400.0, 500.0, 600.0, 700.0, 800.0]
    o = _oracle(dict(random_seed=1, stage_mask=CL, simulation_cluster=1.0), pos,
                clusters=[-1, math.nan, 2.5, math.inf])
    o.step(1)
    assert np.array_equal(o.get_point_positions(), np.asarray(pos, dtype=np.float32))
    assert o.get_cluster_positions().size == 2   # no valid index: clusterCount 1


def test_length_mismatch_ignores_clusters():
    pos = [100.0, 200.0, 300.0, 400.0]
    o = _oracle(dict(random_seed=1, stage_mask=CL, simulation_cluster=1.0), pos, clusters=[0, 0, 0])
    o.step(1)
    assert np.array_equal(o.get_point_positions(), np.asarray(pos, dtype=np.float32))
    assert o.get_cluster_positions().size == 0


def test_strength_scales_the_pull():
    pos = [100.0, 100.0, 300.0, 100.0]
    fields = dict(random_seed=1, stage_mask=CL, simulation_cluster=0.5, simulation_friction=1.0)
    a = _oracle(fields, pos, clusters=[0, 0])
    b = _oracle(fields, pos, clusters=[0, 0], strength=[0.0, 2.0])
    a.step(1)
    b.step(1)
    pa, pb = a.get_point_positions(), b.get_point_positions()
    assert pa[0] == 150.0 and pa[2] == 250.0          # halfway at alpha 1, cluster 0.5
    assert pb[0] == 100.0 and pb[2] == 200.0          # strength 0 stays; strength 2 reaches the centre


# ----------------------------------------------------------------------- GPU --
def _run(eng, orc, ticks, what):
    for t in range(ticks):
        eng.step(1)
        orc.step(1)
        a, b = eng.get_point_positions(), orc.get_point_positions()
        assert same_bits(a, b), (what, t, first_mismatch(a, b))
    ce, co = eng.get_cluster_positions(), orc.get_cluster_positions()
    assert ce.size == co.size and np.array_equal(np.isnan(ce), np.isnan(co))
    assert np.array_equal(ce[~np.isnan(ce)], co[~np.isnan(co)]), what


@pytest.mark.gpu
@pytest.mark.parametrize("k", [1, 7, 256, 257, 5000])
def test_clusters_bit_exact(k):
    pos, links, fields = scenario("ba_small")
    n = pos.size // 2
    rng = np.random.default_rng(k)
    pos = pos.copy()
    pos[2 * 11: 2 * 14] = np.nan                       # absent points
    cl = rng.integers(0, k, size=n).astype(np.float32)
    cl[rng.random(n) < 0.1] = np.nan                   # unclustered
    cl[5] = -3.0
    cp = rng.uniform(500, 3500, size=2 * k).astype(np.float32)
    cp[rng.random(2 * k) < 0.5] = np.nan               # half the coordinates: centre of mass
    st = rng.uniform(0.2, 2.0, size=n).astype(np.float32)
    eng, orc = make_pair(pos, links, dict(fields, simulation_cluster=0.3), pinned=[0, 1, 77], clusters=cl,
                         cluster_positions=cp, cluster_strength=st)
    _run(eng, orc, 8, ("k", k))


@pytest.mark.gpu
def test_cluster_positions_only():
    pos, links, fields = scenario("collision")
    eng, orc = make_pair(pos, links, fields, cluster_positions=[1000.0, 1000.0])
    _run(eng, orc, 4, "positions only")


@pytest.mark.gpu
def test_clusters_alone_and_reset():
    pos, links, fields = scenario("center")
    n = pos.size // 2
    cl = (np.arange(n) % 3).astype(np.float32)
    eng, orc = make_pair(pos, links, dict(fields, stage_mask=CL, simulation_cluster=0.8), clusters=cl)
    _run(eng, orc, 3, "alone")
    for e in (eng, orc):           # clearing the clusters stops the pass
        e.set_point_clusters(None)
        e.render()
    _run(eng, orc, 2, "cleared")
    p0 = eng.get_point_positions()
    eng.step(1)
    assert np.array_equal(eng.get_point_positions(), p0)


@pytest.mark.gpu
def test_clusters_half_million_points():
    n = 500_000
    pos = generators.uniform_positions(n, 0, 8192, 5)
    links = generators.erdos_renyi(n, 6, 5)
    rng = np.random.default_rng(5)
    cl = rng.integers(0, 64, size=n).astype(np.float32)
    eng, orc = make_pair(pos, links, dict(space_size=8192, simulation_repulsion=0.1, simulation_link_distance=2.0,
                                          random_seed=5), clusters=cl)
    _run(eng, orc, 2, "500k")

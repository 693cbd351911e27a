"""Link lists built on the device (ingest_device.cu) against the host build
and the oracle: same rows, order, random draws, bias and strength, so the
layouts agree bit for bit."""
import math

import numpy as np
import pytest

from graph_gb300 import _abi, generators

from helpers import first_mismatch, make_pair, same_bits, scenario

pytestmark = pytest.mark.gpu


def _awkward_links(n, seed):
    rng = np.random.default_rng(seed)
    links = generators.erdos_renyi(n, 6, seed).reshape(-1, 2)
    hub = np.stack([np.zeros(700), rng.integers(1, n, 700)], axis=1)            # a list longer than 256
    loops = np.stack([np.arange(5), np.arange(5)], axis=1)                       # self-loops
    dup = links[:50]                                                             # duplicates
    bad = np.array([[math.nan, 1], [2, -1], [3, n], [4.5, 6], [math.inf, 2], [-0.0, 7], [8, 2.0 ** 40]])
    all_links = np.concatenate([links, hub, loops, dup, bad]).astype(np.float32)
    rng.shuffle(all_links)
    return all_links.reshape(-1)


def _pair(pos, links, fields, dmin, **kw):
    from graph_gb300.engine import Engine
    e = Engine(_abi.make_config(**dict(fields, device_ingest_min_links=dmin)))
    e.set_point_positions(pos)
    e.set_links(links)
    for k, v in kw.items():
        getattr(e, k)(v)
    e.render()
    e.start(1.0)
    return e


STREAMS = [_abi.RANDOM_REFERENCE, _abi.RANDOM_COUNTER]


@pytest.mark.parametrize("stream", STREAMS)
@pytest.mark.parametrize("with_strength", [False, True])
def test_device_and_host_builds_agree(with_strength, stream):
    pos, _, fields = scenario("ba_small")
    fields = dict(fields, random_stream=stream)
    n = pos.size // 2
    pos = pos.copy()
    pos[2 * 9: 2 * 12] = np.nan                      # links to absent points keep their draws
    links = _awkward_links(n, 3)
    kw = {}
    if with_strength:
        s = np.random.default_rng(4).uniform(0, 2, size=links.size // 2).astype(np.float32)
        s[::17] = np.nan
        s[::23] = -1.0
        kw["set_link_strength"] = s
    dev = _pair(pos, links, fields, 0.0, **kw)
    host = _pair(pos, links, fields, math.inf, **kw)
    ld, lh = dev.layout(), host.layout()
    assert (ld.link_entries_in, ld.max_degree_in, ld.max_degree_out) == (lh.link_entries_in, lh.max_degree_in,
                                                                         lh.max_degree_out)
    assert ld.max_degree_in > 256
    assert dev.state().rng_draws == host.state().rng_draws
    for t in range(4):
        dev.step(1)
        host.step(1)
        a, b = dev.get_point_positions(), host.get_point_positions()
        assert same_bits(a, b), (t, first_mismatch(a, b))


@pytest.mark.parametrize("stream", STREAMS)
def test_device_build_matches_oracle(stream):
    pos, _, fields = scenario("collision")
    n = pos.size // 2
    links = _awkward_links(n, 5)
    eng, orc = make_pair(pos, links, dict(fields, device_ingest_min_links=0.0, random_stream=stream))
    for t in range(3):
        eng.step(1)
        orc.step(1)
        a, b = eng.get_point_positions(), orc.get_point_positions()
        assert same_bits(a, b), (t, first_mismatch(a, b))


def test_device_build_edge_cases():
    pos, _, fields = scenario("center")
    n = pos.size // 2
    for links in (np.array([math.nan, 1.0, 5.0, -2.0], dtype=np.float32),     # no valid link
                  np.array([0.0, 1.0], dtype=np.float32),                     # one link
                  np.tile(np.array([3.0, 4.0], dtype=np.float32), 300)):      # one row of 300 duplicates
        eng, orc = make_pair(pos, links, dict(fields, device_ingest_min_links=0.0))
        eng.step(2)
        orc.step(2)
        a, b = eng.get_point_positions(), orc.get_point_positions()
        assert same_bits(a, b), first_mismatch(a, b)
        assert eng.state().rng_draws == orc.state().rng_draws

"""A render that the device-memory budget refuses part way leaves no
half-built graph behind: the engine forgets the graph (0 points, nothing to
tick or read) and rewinds the random stream, and a later render with room
builds it again, bit-exact with an uninterrupted run."""
import numpy as np
import pytest

from graph_gb300 import _abi, generators
from graph_gb300._calls import StatusError
from graph_gb300.engine import Engine
from oracle import OracleEngine

pytestmark = pytest.mark.gpu

FIELDS = dict(space_size=4096.0, simulation_repulsion=0.3, simulation_link_distance=2.0, random_seed=5)


def _same(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_refused_render_forgets_the_graph_and_a_retry_rebuilds_it():
    small = generators.centred_square(1000, 4096, 5)
    big = generators.centred_square(200_000, 4096, 6)
    links = generators.erdos_renyi(200_000, 4, 6)
    eng = Engine(**dict(FIELDS, hbm_budget_bytes=40e6))
    try:
        eng.set_point_positions(small)
        eng.render()
        eng.start(1.0)
        eng.step(2)
        assert eng.layout().points_number == 1000
        # the larger graph needs more than 40 MB: the render is refused part way
        eng.set_point_positions(big)
        eng.set_links(links)
        with pytest.raises(StatusError) as e:
            eng.render()
        assert e.value.status == _abi.CGL_OOM
        lay = eng.layout()
        assert lay.points_number == 0 and lay.levels == 0   # forgotten before anything can tick
        eng.step(3)                                            # nothing to tick
        assert eng.get_point_positions().size == 0
        # room again: the staged graph is built from scratch
        eng.set_config(_abi.make_config(**dict(FIELDS, hbm_budget_bytes=0.0)))
        eng.render()
        eng.start(1.0)
        eng.step(3)
        got = eng.get_point_positions()
    finally:
        eng.close()
    # the oracle takes the same successful renders and ticks: the refused render draws nothing
    orc = OracleEngine(_abi.make_config(**FIELDS))
    orc.set_point_positions(small)
    orc.render()
    orc.start(1.0)
    orc.step(2)
    orc.set_point_positions(big)
    orc.set_links(links)
    orc.render()
    orc.start(1.0)
    orc.step(3)
    want = orc.get_point_positions()
    orc.close()
    assert _same(got, want)

"""The seeded synthetic workloads (graph_gb300/generators.py) that stand in
for datasets: same seed, same arrays; the documented shapes hold."""
import numpy as np

from graph_gb300 import generators


def _pairs(links):
    return np.asarray(links, np.float64).reshape(-1, 2).astype(np.int64)


def _check_simple(pairs, n, directed=False):
    assert pairs.min() >= 0 and pairs.max() < n
    assert np.all(pairs[:, 0] != pairs[:, 1])                                  # no self-loops
    if directed:                                                               # no repeated (source, target)
        key = pairs[:, 0] * n + pairs[:, 1]
    else:                                                                      # no repeated pair either way
        key = np.minimum(pairs[:, 0], pairs[:, 1]) * n + np.maximum(pairs[:, 0], pairs[:, 1])
    assert np.unique(key).size == key.size


def test_same_seed_same_arrays():
    for make in (lambda s: generators.barabasi_albert(500, 3, s),
                 lambda s: generators.erdos_renyi(500, 6, s),
                 lambda s: generators.sbm_zipf(2000, 20, 1.2, 10, 0.9, s),
                 lambda s: generators.rmat(10, 5000, 0.57, 0.19, 0.19, s),
                 lambda s: generators.preferential_attachment(500, 4, s),
                 lambda s: generators.centred_square(300, 4096, s)):
        a, b, c = make(1), make(1), make(2)
        assert np.array_equal(a, b)
        assert not np.array_equal(a, c)


def test_erdos_renyi_edge_count():
    links = generators.erdos_renyi(1000, 6, 3)
    pairs = _pairs(links)
    assert pairs.shape[0] == 3000
    _check_simple(pairs, 1000)


def test_barabasi_albert_links_to_distinct_earlier_points():
    n, m = 800, 4
    pairs = _pairs(generators.barabasi_albert(n, m, 5))
    assert pairs.min() >= 0 and pairs.max() < n
    assert np.all(pairs[:, 0] != pairs[:, 1])
    deg = np.bincount(pairs.reshape(-1), minlength=n)
    assert deg.max() > 5 * m                                                   # preferential attachment makes hubs


def test_rmat_and_sbm_are_simple_graphs():
    pairs = _pairs(generators.rmat(11, 8000, 0.57, 0.19, 0.19, 7))
    _check_simple(pairs, 1 << 11, directed=True)
    assert 0.9 * 8000 <= pairs.shape[0] <= 8000
    n = 5000
    pairs = _pairs(generators.sbm_zipf(n, 50, 1.2, 10, 0.9, 8))
    _check_simple(pairs, n)
    assert 0.8 * n * 10 / 2 <= pairs.shape[0] <= n * 10 / 2


def test_centred_square_bounds():
    pos = generators.centred_square(10000, 4096, 9)
    assert pos.dtype == np.float32 and pos.size == 20000
    assert pos.min() >= 4096 * 3 / 8 and pos.max() <= 4096 * 5 / 8


def test_batch_workload_jobs():
    jobs = list(generators.batch_workload(8, 11, n_min=100, n_max=2000))
    assert len(jobs) == 8
    for pos, links, fields in jobs:
        n = pos.size // 2
        assert 100 <= n <= 2000
        assert fields["space_size"] in [2.0 ** k for k in range(9, 15)]
        assert 0.05 <= fields["simulation_repulsion"] <= 0.5
        pairs = _pairs(links)
        assert pairs.min() >= 0 and pairs.max() < n

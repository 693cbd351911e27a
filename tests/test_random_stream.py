"""The reference's random stream (random@4.1.0 over seedrandom@3.0.5), on CPU.

Three restatements are checked against seedrandom's published known answers
and against each other: the product's (graph_gb300/csrc/random_stream.h,
called through cgl_random_draws, which needs no GPU), the oracle's
(oracle/oracle.cpp) and a pure-Python one (tests/seedrandom_ref.py).  Then the
oracle's jitter and link rest-length draws for randomSeed = 1 are derived from
the stream in the reference's order: ForceManyBody.create's two draws per texel
(ForceManyBody/index.ts:133-138), ForceLink.create's one draw per list entry,
incoming lists first (ForceLink/index.ts:76, src/index.ts:1663-1666), and one
near-field seed per tick (ForceManyBody/index.ts:521).
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from graph_gb300 import _abi, generators
from oracle import OracleEngine

from seedrandom_ref import SeedRandom

# seedrandom's README: `new Math.seedrandom('hello.')` gives these two doubles,
# then quick() and int32() give 0.7316977467853576 and 1966374204.
README_SEED = "hello."
README_FIRST = [0.9282578795792454, 0.3752569768646784]

SEEDS = ["1", "0", "42", "", "hello.", "-7", "1.5", "seed with spaces", "é中\U0001F600", "x" * 300,
         "".join(chr(33 + (k * 7) % 90) for k in range(257))]


def product_draws(lib, seed, n):
    out = np.zeros(n, dtype=np.float64)
    st = lib.cgl_random_draws(seed.encode("utf-8"), n, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == _abi.CGL_OK
    return out


def test_readme_known_answers_python():
    r = SeedRandom(README_SEED)
    assert [r.next(), r.next()] == README_FIRST
    assert r.g(4) / 2.0 ** 32 == 0.7316977467853576
    v = r.g(4)
    assert (v - 2 ** 32 if v >= 2 ** 31 else v) == 1966374204


def test_readme_known_answers_oracle():
    assert oracle.seedrandom(README_SEED, 2).tolist() == README_FIRST


def test_readme_known_answers_product(engine_lib):
    assert product_draws(engine_lib, README_SEED, 2).tolist() == README_FIRST


@pytest.mark.parametrize("seed", SEEDS)
def test_three_restatements_agree(engine_lib, seed):
    n = 3000 if len(seed) < 5 else 300
    want = SeedRandom(seed)
    want = np.array([want.next() for _ in range(n)])
    assert np.array_equal(oracle.seedrandom(seed, n), want)
    assert np.array_equal(product_draws(engine_lib, seed, n), want)


def test_long_stream_agrees(engine_lib):
    # 200k draws cover the rare doubles that take more than 7 bytes
    a = product_draws(engine_lib, "1", 200_000)
    b = oracle.seedrandom("1", 200_000)
    assert np.array_equal(a, b)
    assert a.min() >= 0 and a.max() < 1


def test_jitter_and_rest_lengths_for_seed_1():
    # a small graph, randomSeed = 1: every jitter value and rest-length draw is
    # the stream's value at its place in the reference's order
    n = 50
    pos = generators.uniform_positions(n, 0, 4096, 1)
    links = np.array([0, 1, 1, 2, 2, 0, 7, 3, 3, 7, 9, 4, 4, 9, 60, 1, 2.5, 3, 8, 8], dtype=np.float32)
    o = OracleEngine(random_seed=1)
    o.set_point_positions(pos)
    o.set_links(links)
    o.render()
    r = SeedRandom("1")
    t = math.ceil(math.sqrt(n))
    jit = []
    for texel in range(t * t):
        x = np.float32(r.float(-1, 1) * 0.00001)
        y = np.float32(r.float(-1, 1) * 0.00001)
        if texel < n:
            jit += [x, y]
    assert np.array_equal(o.jitter(), np.array(jit, dtype=np.float32))
    for direction in (0, 1):
        c = o.csr(direction)
        want = np.array([np.float32(r.float(0, 1)) for _ in range(c["col"].size)], dtype=np.float32)
        assert c["col"].size == 8
        assert np.array_equal(c["rnd"], want), direction
    o.start()
    o.step(3)   # three peel seeds
    assert o.state().rng_draws == 2 * t * t + 16 + 3


def test_string_and_float_seeds_use_their_text():
    # randomSeed may be a string or any number; the stream is keyed by String(seed)
    for seed, text in (("abc", "abc"), (1.5, "1.5"), (-3, "-3"), (2.0, "2"), (1e21, "1e+21"), (1e-7, "1e-7"),
                       (123456789.125, "123456789.125")):
        u64, t = _abi.seed_fields(seed)
        got = t if t is not None else str(u64)
        assert got == text, (seed, got)
        o = OracleEngine(random_seed=seed)
        o.set_point_positions(np.array([10.0, 10.0], dtype=np.float32))
        o.render()
        want = np.float32(SeedRandom(text).float(-1, 1) * 0.00001)
        assert o.jitter()[0] == want, seed


def test_js_number_to_string():
    cases = {0.1: "0.1", 100.0: "100", 1e21: "1e+21", 1.5e-7: "1.5e-7", 123e-20: "1.23e-18", 0.000001: "0.000001",
             1.7976931348623157e308: "1.7976931348623157e+308", -2.5: "-2.5", 5e-324: "5e-324",
             123456789012345680000.0: "123456789012345680000"}
    for x, want in cases.items():
        assert _abi.js_number_to_string(x) == want, x


def test_counter_stream_is_opt_in():
    pos = generators.uniform_positions(100, 0, 4096, 2)
    a = OracleEngine(random_seed=5)
    b = OracleEngine(random_seed=5, random_stream=_abi.RANDOM_COUNTER)
    for e in (a, b):
        e.set_point_positions(pos)
        e.render()
    u = SeedRandom("5").next()
    assert a.jitter()[0] == np.float32((u * 2 - 1) * 1e-5)
    c0 = (oracle.splitmix_draw(5, 0) >> 11) * 2.0 ** -53
    assert b.jitter()[0] == np.float32((c0 * 2 - 1) * 1e-5)

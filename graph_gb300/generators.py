"""Seeded synthetic graph generators for the benchmark workloads.

The reference benchmarks on generated data only (src/stories/performance/
repulsion-benchmark.ts:29-37, unseeded Math.random); these generators are the
project's own, seeded with numpy's PCG64, and produce float32 source/target
pairs in the reference's `setLinks` layout.
"""
import numpy as np


def barabasi_albert(n, m, seed):
    """Barabasi-Albert preferential attachment: each new point links to m distinct earlier points."""
    rng = np.random.default_rng(seed)
    m = int(m)
    src = []
    dst = []
    rep = np.zeros(2 * m * n + m, dtype=np.int64)   # endpoint multiset: degree-proportional sampling
    used = 0
    for v in range(m, n):
        if used == 0:
            chosen = list(range(m))
        else:
            chosen = []
            seen = set()
            while len(chosen) < m:
                for p in rep[rng.integers(0, used, size=2 * (m - len(chosen)))]:
                    p = int(p)
                    if p not in seen:
                        seen.add(p)
                        chosen.append(p)
                        if len(chosen) == m:
                            break
        for t in chosen:
            src.append(v)
            dst.append(t)
        rep[used:used + m] = chosen
        rep[used + m:used + 2 * m] = v
        used += 2 * m
    links = np.empty(2 * len(src), dtype=np.float32)
    links[0::2] = src
    links[1::2] = dst
    return links


def erdos_renyi(n, mean_degree, seed):
    """G(n, M) with M = n * mean_degree / 2 distinct non-loop edges."""
    rng = np.random.default_rng(seed)
    m = int(round(n * mean_degree / 2))
    s = rng.integers(0, n, size=int(m * 1.2) + 16, dtype=np.int64)
    t = rng.integers(0, n, size=s.size, dtype=np.int64)
    keep = s != t
    s, t = s[keep], t[keep]
    key = np.minimum(s, t) * n + np.maximum(s, t)
    _, first = np.unique(key, return_index=True)
    first = np.sort(first)[:m]
    links = np.empty(2 * first.size, dtype=np.float32)
    links[0::2] = s[first]
    links[1::2] = t[first]
    return links


def sbm_zipf(n, communities, zipf_s, mean_degree, intra_fraction, seed):
    """Stochastic block model with Zipf(s) community sizes.

    Draws n*mean_degree/2 links; a fraction `intra_fraction` joins two points of
    the same community (community chosen proportional to its size squared, the
    SBM's intra-pair weight), the rest join points of different communities.
    Self-loops and duplicates are dropped.
    """
    rng = np.random.default_rng(seed)
    w = 1.0 / np.arange(1, communities + 1) ** zipf_s
    sizes = np.maximum(1, np.floor(w / w.sum() * n)).astype(np.int64)
    sizes[0] += n - sizes.sum()
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    perm = rng.permutation(n)   # community members spread over the index space
    m = int(round(n * mean_degree / 2))
    m_in = int(round(m * intra_fraction))
    m_out = m - m_in
    over = 1.05
    pw = sizes.astype(np.float64) ** 2
    pw /= pw.sum()
    c = rng.choice(communities, size=int(m_in * over) + 16, p=pw)
    a = starts[c] + (rng.random(c.size) * sizes[c]).astype(np.int64)
    b = starts[c] + (rng.random(c.size) * sizes[c]).astype(np.int64)
    s_out = rng.integers(0, n, size=int(m_out * over) + 16)
    t_out = rng.integers(0, n, size=s_out.size)
    comm_of = np.repeat(np.arange(communities), sizes)
    keep = comm_of[s_out] != comm_of[t_out]
    s_out, t_out = s_out[keep], t_out[keep]
    s = np.concatenate([a, s_out])
    t = np.concatenate([b, t_out])
    keep = s != t
    s, t = s[keep], t[keep]
    key = np.minimum(s, t) * n + np.maximum(s, t)
    _, first = np.unique(key, return_index=True)
    first = np.sort(first)
    intra = first[first < a.size][:m_in]
    inter = first[first >= a.size][:m_out]
    sel = np.sort(np.concatenate([intra, inter]))
    s, t = perm[s[sel]], perm[t[sel]]
    links = np.empty(2 * s.size, dtype=np.float32)
    links[0::2] = s
    links[1::2] = t
    return links


def rmat(scale, n_edges, a, b, c, seed):
    """R-MAT (Chakrabarti et al. 2004) edges on 2^scale points; self-loops and duplicates removed."""
    rng = np.random.default_rng(seed)
    n = 1 << scale
    target = int(n_edges)
    out_s = np.zeros(0, dtype=np.int64)
    out_t = np.zeros(0, dtype=np.int64)
    draw = int(target * 1.15) + 1024
    while True:
        s = np.zeros(draw, dtype=np.int64)
        t = np.zeros(draw, dtype=np.int64)
        for _ in range(scale):
            r = rng.random(draw)
            sb = (r >= a + b).astype(np.int64)                    # quadrants c, d set the source bit
            tb = ((r >= a) & (r < a + b) | (r >= a + b + c)).astype(np.int64)
            s = (s << 1) | sb
            t = (t << 1) | tb
        keep = s != t
        out_s = np.concatenate([out_s, s[keep]])
        out_t = np.concatenate([out_t, t[keep]])
        key = out_s * n + out_t
        _, first = np.unique(key, return_index=True)
        first = np.sort(first)
        out_s, out_t = out_s[first], out_t[first]
        if out_s.size >= target:
            break
        draw = int((target - out_s.size) * 1.5) + 1024
    out_s, out_t = out_s[:target], out_t[:target]
    links = np.empty(2 * out_s.size, dtype=np.float32)
    links[0::2] = out_s
    links[1::2] = out_t
    return links


def uniform_positions(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=2 * n).astype(np.float32)


def centred_square(n, space, seed):
    """Uniform in the centred square of side space/4."""
    return uniform_positions(n, space * 3 / 8, space * 5 / 8, seed)


def preferential_attachment(n, m, seed):
    """Barabasi-Albert-style graph by edge copying (Batagelj & Brandes 2005), vectorised.

    Node v >= m adds m edges; each target is an endpoint drawn uniformly from
    all endpoints of earlier edges (degree-proportional), resolved by pointer
    jumping.  Self-loops and duplicate pairs are dropped, so a node keeps at
    most m edges.
    """
    rng = np.random.default_rng(seed)
    m = int(m)
    if n <= m:
        return np.zeros(0, dtype=np.float32)
    k = np.arange(m * (n - m), dtype=np.int64)          # edge index
    src = m + k // m
    # endpoints: 2k = source of edge k, 2k+1 = target of edge k; the first m
    # edges (node m) attach to nodes 0..m-1 directly
    ptr = (rng.random(k.size) * (2 * k)).astype(np.int64)
    tgt = np.full(k.size, -1, dtype=np.int64)
    first = k < m
    tgt[first] = k[first]
    ptr[first] = -1
    even = (~first) & (ptr % 2 == 0)
    tgt[even] = src[ptr[even] // 2]
    todo = np.nonzero(tgt < 0)[0]
    ref = ptr[todo] // 2                                 # points at the target of an earlier edge
    while todo.size:
        t = tgt[ref]
        done = t >= 0
        tgt[todo[done]] = t[done]
        todo, ref = todo[~done], ptr[ref[~done]]
        odd = ref % 2 == 1
        # ref now holds raw endpoint positions; even ones are sources
        res = np.where(odd, -1, src[np.maximum(ref, 0) // 2])
        hit = ~odd
        tgt[todo[hit]] = res[hit]
        todo, ref = todo[~hit], ref[~hit] // 2
    keep = tgt != src
    s, t = src[keep], tgt[keep]
    key = np.minimum(s, t) * n + np.maximum(s, t)
    _, first_idx = np.unique(key, return_index=True)
    first_idx = np.sort(first_idx)
    links = np.empty(2 * first_idx.size, dtype=np.float32)
    links[0::2] = s[first_idx]
    links[1::2] = t[first_idx]
    return links


def batch_workload(count, seed, n_min=100, n_max=100_000):
    """Independent layout jobs: sizes log-uniform over [n_min, n_max], half
    preferential-attachment (m in 2..6) and half Erdos-Renyi (mean degree in
    4..12), each with its own seed, a power-of-two spaceSize fitted to its size
    (2^round(log2(41 sqrt(n))), within [512, 16384]) and repulsion drawn from
    [0.05, 0.5]; positions uniform in the centred square of side spaceSize/4.
    Yields (positions, links, config fields)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count)).astype(np.int64)
    for g in range(count):
        n = int(sizes[g])
        gseed = int(rng.integers(0, 2**31))
        if g % 2 == 0:
            links = preferential_attachment(n, int(rng.integers(2, 7)), gseed)
        else:
            links = erdos_renyi(n, float(rng.uniform(4, 12)), gseed)
        space = float(2 ** int(np.clip(np.round(np.log2(41 * np.sqrt(n))), 9, 14)))
        pos = centred_square(n, space, gseed + 1)
        fields = dict(space_size=space, simulation_repulsion=float(rng.uniform(0.05, 0.5)),
                      simulation_gravity=0.25, simulation_friction=0.85, simulation_link_spring=1.0,
                      simulation_link_distance=2.0, simulation_decay=5000, random_seed=gseed)
        yield pos, links, fields

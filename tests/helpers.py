"""Shared scenario builders for the oracle and engine tests."""
import numpy as np

from graph_gb300 import _abi, generators


def scenario(kind, seed=1):
    """Return (positions, links, config fields) for a named small workload."""
    if kind == "ba_small":
        n = 2000
        return (generators.centred_square(n, 4096, seed), generators.barabasi_albert(n, 5, seed),
                dict(space_size=4096, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                     simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_decay=5000,
                     random_seed=seed))
    if kind == "cfg0":
        # Barabasi-Albert N=10,000, m=5, centred square of side S/4, S=4096
        n = 10000
        return (generators.centred_square(n, 4096, seed), generators.barabasi_albert(n, 5, seed),
                dict(space_size=4096, simulation_repulsion=0.1, simulation_gravity=0.25, simulation_friction=0.85,
                     simulation_link_spring=1.0, simulation_link_distance=2.0, simulation_decay=5000,
                     random_seed=seed))
    if kind == "dense":
        # many points in few finest cells: exercises the 8-slot peel and hub cells
        n = 3000
        rng = np.random.default_rng(seed)
        pos = (2048 + rng.normal(0, 30, size=2 * n)).astype(np.float32)
        links = generators.erdos_renyi(n, 6, seed)
        return pos, links, dict(space_size=4096, simulation_repulsion=1.0, random_seed=seed)
    if kind == "collision":
        n = 4000
        rng = np.random.default_rng(seed)
        pos = rng.uniform(1800, 2300, size=2 * n).astype(np.float32)
        links = generators.erdos_renyi(n, 4, seed)
        return pos, links, dict(space_size=4096, simulation_collision=0.5, simulation_repulsion=0.5,
                                simulation_link_distance=2.0, random_seed=seed)
    if kind == "center":
        n = 1500
        pos = generators.uniform_positions(n, 100, 3000, seed)
        links = generators.erdos_renyi(n, 4, seed)
        return pos, links, dict(space_size=4096, simulation_center=0.5, simulation_gravity=0.1, random_seed=seed)
    raise KeyError(kind)


def make_pair(pos, links, fields, extra=None, sizes=None, strength=None, pinned=None, clusters=None,
              cluster_positions=None, cluster_strength=None):
    """Engine and oracle with identical staged data, rendered and started."""
    from graph_gb300.engine import Engine
    from oracle import OracleEngine
    cfg = _abi.make_config(**fields)
    pair = []
    for cls in (Engine, OracleEngine):
        e = cls(cfg)
        e.set_point_positions(pos)
        if links is not None:
            e.set_links(links)
        if strength is not None:
            e.set_link_strength(strength)
        if sizes is not None:
            e.set_point_sizes(sizes)
        if pinned is not None:
            e.set_pinned_points(pinned)
        if clusters is not None:
            e.set_point_clusters(clusters)
        if cluster_positions is not None:
            e.set_cluster_positions(cluster_positions)
        if cluster_strength is not None:
            e.set_point_cluster_strength(cluster_strength)
        e.render()
        e.start(1.0)
        pair.append(e)
    return pair


def same_bits(a, b):
    """Bitwise equality of two float32 arrays, treating all NaNs alike."""
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def first_mismatch(a, b):
    a = np.asarray(a, dtype=np.float32).reshape(-1)
    b = np.asarray(b, dtype=np.float32).reshape(-1)
    bad = np.nonzero(~((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))[0]
    if bad.size == 0:
        return None
    i = int(bad[0])
    return dict(count=int(bad.size), index=i, a=float(a[i]), b=float(b[i]))


def mass_seen(cells_by_level, pos, space, absent=None):
    """Per point, the number of points its level passes and near field account for.

    Re-applies the reference's coverage rule (force-level.frag:70-95,
    force-nearfield.frag:213-223) to the retained cell counts; for every live
    point the total must be live - 1 (exactly-once tiling,
    docs/many-body-force/README.md:74-87).
    """
    L = len(cells_by_level)
    gf = 4 << (L - 1)
    n = pos.size // 2
    x = pos[0::2].astype(np.float32)
    y = pos[1::2].astype(np.float32)
    csf = np.float32(space / gf)
    fcx = np.clip(np.floor(x / csf), 0, gf - 1).astype(np.int64)
    fcy = np.clip(np.floor(y / csf), 0, gf - 1).astype(np.int64)
    seen = np.zeros(n, dtype=np.float64)
    for l in range(L):
        g = 4 << l
        cnt = cells_by_level[l][..., 2]   # [g, g] indexed [y, x]
        sh = L - 1 - l
        pcx, pcy = fcx >> sh, fcy >> sh
        if l == 0:
            for j in range(g):
                for i in range(g):
                    far = np.maximum(np.abs(i - pcx), np.abs(j - pcy)) > 1
                    seen += np.where(far, cnt[j, i], 0)
        else:
            bx, by = (pcx // 2) * 2 - 2, (pcy // 2) * 2 - 2
            for j in range(6):
                for i in range(6):
                    cx, cy = bx + i, by + j
                    ok = (cx >= 0) & (cy >= 0) & (cx < g) & (cy < g)
                    far = np.maximum(np.abs(cx - pcx), np.abs(cy - pcy)) > 1
                    v = cnt[np.clip(cy, 0, g - 1), np.clip(cx, 0, g - 1)]
                    seen += np.where(ok & far, v, 0)
    fine = cells_by_level[L - 1][..., 2]
    for j in (-1, 0, 1):
        for i in (-1, 0, 1):
            cx, cy = fcx + i, fcy + j
            ok = (cx >= 0) & (cy >= 0) & (cx < gf) & (cy < gf)
            v = fine[np.clip(cy, 0, gf - 1), np.clip(cx, 0, gf - 1)] - (1 if (i == 0 and j == 0) else 0)
            seen += np.where(ok, v, 0)
    if absent is not None:
        seen[absent] = np.nan
    return seen

"""Generate tests/golden/golden.json: known answers for tiny simulations.

Each case is worked out here from the reference's formulas in plain FP64
Python, independently of the C++ oracle (which computes in FP32): gravity
(force-gravity.frag:24-40), center (force-center.frag:22-36), a linked pair
(force-spring.ts:38-96, ForceLink/index.ts:40-83), a repelling pair resolved
by the near field alone (force-nearfield.frag:64-263), an overlapping
collision pair (force-collision-spatial.frag:103-168), and the cluster pull
towards a centre of mass or a given cluster position (force-cluster.frag:28-53,
calculate-centermass.vert:22-52).  The update is
update-position.frag:52-57 and alpha follows Store/index.ts:328-332.  Random
draws are the reference's stream (random@4.1.0 over seedrandom@3.0.5, restated
in tests/seedrandom_ref.py) in the reference's order.
Run:  python tests/golden/make_golden.py
"""
import json
import math
import os

import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from seedrandom_ref import SeedRandom  # noqa: E402

STAGE = dict(gravity=1, center=2, manybody=4, link_in=8, link_out=16, collision=32, clusters=64)


def unit(seed, k):
    """Draw k (0-based) of the reference's stream for randomSeed = seed."""
    r = SeedRandom(str(seed))
    for _ in range(k):
        r.next()
    return r.next()


def alpha_next(a, decay=5000):
    return a + (0 - a) * (1 - math.pow(0.001, 1 / decay))


def clamp(v, lo, hi):
    return min(max(v, lo), hi)


def case_gravity():
    S, g, fr = 4096.0, 0.25, 0.85
    p = [1000.0, 3000.0]
    a = 1.0
    for _ in range(3):
        c = S / 2
        dx, dy = c - p[0], c - p[1]
        # alpha*g*dist*0.1 * unit vector = alpha*g*0.1 * d
        p = [clamp(p[0] + fr * a * g * 0.1 * dx, 0, S), clamp(p[1] + fr * a * g * 0.1 * dy, 0, S)]
        a = alpha_next(a)
    return dict(name="gravity_single", config=dict(random_seed=11, stage_mask=STAGE["gravity"]),
                positions=[1000.0, 3000.0], links=[], ticks=3, expected=p, atol=2e-3)


def case_center():
    S, cf, fr = 4096.0, 0.5, 0.85
    pts = [[1000.0, 1200.0], [2000.0, 2600.0], [1500.0, 900.0]]
    a = 1.0
    for _ in range(2):
        cx = sum(q[0] for q in pts) / 3
        cy = sum(q[1] for q in pts) / 3
        pts = [[clamp(q[0] + fr * a * cf * 0.01 * (cx - q[0]), 0, S),
                clamp(q[1] + fr * a * cf * 0.01 * (cy - q[1]), 0, S)] for q in pts]
        a = alpha_next(a)
    flat = [v for q in pts for v in q]
    return dict(name="center_triple", config=dict(random_seed=12, simulation_center=0.5, stage_mask=STAGE["center"]),
                positions=[1000.0, 1200.0, 2000.0, 2600.0, 1500.0, 900.0], links=[], ticks=2, expected=flat,
                atol=2e-3)


def case_link_pair():
    seed, S, fr, dist, spring = 13, 4096.0, 0.85, 2.0, 1.0
    r0, r1 = 1.0, 1.2
    p = [[2000.0, 2000.0], [2010.0, 2003.0]]
    # draws: jitter 2*T^2 = 8 (T = 2), then the incoming entry (point 0 -> 1), then the outgoing one
    rin, rout = unit(seed, 8), unit(seed, 9)
    bias, strength = 0.5, 1.0
    a = 1.0

    def spring_v(pp, q, r):
        d = (r * (r1 - r0) + r0) * dist
        x, y = q[0] - pp[0], q[1] - pp[1]
        l = math.hypot(x, y)
        l = max(l, d * 0.99)
        f = (l - d) / l * spring * a * strength * bias
        return [x * f, y * f]

    for _ in range(2):
        v = spring_v(p[0], p[1], rin)
        p[0] = [clamp(p[0][0] + fr * v[0], 0, S), clamp(p[0][1] + fr * v[1], 0, S)]
        v = spring_v(p[1], p[0], rout)
        p[1] = [clamp(p[1][0] + fr * v[0], 0, S), clamp(p[1][1] + fr * v[1], 0, S)]
        a = alpha_next(a)
    return dict(name="link_pair", config=dict(random_seed=seed, simulation_link_distance=dist,
                                               stage_mask=STAGE["link_in"] | STAGE["link_out"]),
                positions=[2000.0, 2000.0, 2010.0, 2003.0], links=[0, 1], ticks=2,
                expected=[p[0][0], p[0][1], p[1][0], p[1][1]], atol=2e-3)


def case_repulsion_pair():
    seed, S, fr, rep = 14, 4096.0, 0.85, 1.0
    p = [[1000.0, 1000.0], [1003.0, 1004.0]]
    # jitter of point i = draws (2i, 2i+1) scaled U(-1,1) * 1e-5
    jit = [[(unit(seed, 2 * i) * 2 - 1) * 1e-5, (unit(seed, 2 * i + 1) * 2 - 1) * 1e-5] for i in range(2)]
    a = 1.0
    out = []
    for i in range(2):
        o = p[1 - i]
        dx, dy = p[i][0] - o[0], p[i][1] - o[1]
        l = math.hypot(dx, dy)
        add = a * rep / l
        v = [add * dx / l, add * dy / l]
        v = [v[0] + v[0] * jit[i][0], v[1] + v[1] * jit[i][1]]
        out += [clamp(p[i][0] + fr * v[0], 0, S), clamp(p[i][1] + fr * v[1], 0, S)]
    return dict(name="repulsion_pair", config=dict(random_seed=seed, stage_mask=STAGE["manybody"]),
                positions=[1000.0, 1000.0, 1003.0, 1004.0], links=[], ticks=1, expected=out, atol=2e-4)


def case_collision_pair():
    S, fr = 4096.0, 0.85
    p = [[1000.3, 1000.3], [1000.9, 1001.1]]
    # default size 4 -> radius 2, combined 4; each of the 4 offset passes pushes
    # with min(alpha*0.5*sqrt(ov)*4*0.5*0.25, 2), capped at 0.1 * radius = 0.2
    a, strength = 1.0, 0.5
    out = []
    for i in range(2):
        o = p[1 - i]
        dx, dy = p[i][0] - o[0], p[i][1] - o[1]
        dist = math.hypot(dx, dy)
        ov = (4 - dist) / 4
        f = min(a * strength * math.sqrt(ov) * 4 * 0.5 * 0.25, 2.0)
        f = min(f, 0.2)
        v = [4 * f * dx / dist, 4 * f * dy / dist]
        out += [clamp(p[i][0] + fr * v[0], 0, S), clamp(p[i][1] + fr * v[1], 0, S)]
    return dict(name="collision_pair", config=dict(random_seed=15, simulation_collision=0.5,
                                                    stage_mask=STAGE["collision"]),
                positions=[1000.3, 1000.3, 1000.9, 1001.1], links=[], ticks=1, expected=out, atol=2e-4)


def cluster_ticks(pts, of, custom, coeff, cc, ticks, fr=0.85, S=4096.0):
    """alpha*dist*cc*coeff * (d/dist) = alpha*cc*coeff*d towards the cluster's
    given position, else its live members' centre of mass; unclustered points
    only get the update."""
    a = 1.0
    for _ in range(ticks):
        cm = {}
        for k in set(c for c in of if c is not None):
            mem = [q for q, c in zip(pts, of) if c == k]
            cm[k] = (sum(q[0] for q in mem) / len(mem), sum(q[1] for q in mem) / len(mem))
        new = []
        for q, c, w in zip(pts, of, coeff):
            if c is None:
                new.append(q)
                continue
            t = custom.get(c, cm[c])
            new.append([clamp(q[0] + fr * a * cc * w * (t[0] - q[0]), 0, S),
                        clamp(q[1] + fr * a * cc * w * (t[1] - q[1]), 0, S)])
        pts = new
        a = alpha_next(a)
    return [v for q in pts for v in q]


def case_cluster_centroid():
    pos = [[1000.0, 1200.0], [1400.0, 1000.0], [3000.0, 3100.0], [2000.0, 2000.0], [900.0, 1500.0]]
    of = [0, 0, 1, None, 0]
    exp = cluster_ticks(pos, of, {}, [1.0] * 5, 0.5, 3)
    return dict(name="cluster_centroid", config=dict(random_seed=16, simulation_cluster=0.5,
                                                      stage_mask=STAGE["clusters"]),
                positions=[v for q in pos for v in q], links=[], clusters=[0, 0, 1, None, 0], ticks=3,
                expected=exp, atol=2e-3)


def case_cluster_custom():
    pos = [[1000.0, 1200.0], [1400.0, 1000.0], [3000.0, 3100.0], [2000.0, 2000.0]]
    of = [0, 1, 1, 0]
    coeff = [1.0, 0.5, 2.0, 0.25]
    exp = cluster_ticks(pos, of, {0: (500.0, 600.0)}, coeff, 0.1, 2)
    return dict(name="cluster_custom_position", config=dict(random_seed=17, stage_mask=STAGE["clusters"]),
                positions=[v for q in pos for v in q], links=[], clusters=of, cluster_positions=[500.0, 600.0, None, None],
                cluster_strength=coeff, ticks=2, expected=exp, atol=2e-3)


def main():
    cases = [case_gravity(), case_center(), case_link_pair(), case_repulsion_pair(), case_collision_pair(),
             case_cluster_centroid(), case_cluster_custom()]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(dict(generator="tests/golden/make_golden.py", cases=cases), f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()

"""Layout agreement measures for full runs.

Long force-layout trajectories are chaotic: two implementations that differ in
one rounding drift apart after a few hundred ticks, while both still produce a
good layout.  Full runs are therefore compared by shape, not point by point:

* Procrustes-aligned RMS distance: the second layout is translated, rotated
  (and optionally scaled) onto the first by least squares (the orthogonal
  Procrustes solution from the SVD of the centred cross-covariance), then the
  root-mean-square distance between matching points is taken.  `relative`
  divides it by the first layout's RMS radius about its centroid.
* Edge-length stress: sqrt(sum_e (l_a(e) - l_b(e))^2 / sum_e l_a(e)^2) over the
  links, each length taken within its own layout.

Absent points (NaN) are left out of both measures.  All arithmetic is FP64.
"""
import numpy as np


def _xy(a):
    return np.asarray(a, dtype=np.float64).reshape(-1, 2)


def procrustes_rms(a, b, scale=False):
    """(rms, relative) distance between layouts a and b after aligning b onto a."""
    pa, pb = _xy(a), _xy(b)
    live = ~(np.isnan(pa).any(axis=1) | np.isnan(pb).any(axis=1))
    pa, pb = pa[live], pb[live]
    if pa.shape[0] == 0 or np.array_equal(pa, pb):
        return 0.0, 0.0   # identical layouts: exactly 0 (the SVD would leave rounding)
    ca, cb = pa.mean(axis=0), pb.mean(axis=0)
    xa, xb = pa - ca, pb - cb
    u, s, vt = np.linalg.svd(xb.T @ xa)
    d = np.sign(np.linalg.det(u @ vt))
    dm = np.diag([1.0, d])
    r = u @ dm @ vt                       # rotation taking xb onto xa
    k = 1.0
    if scale:
        nb = (xb * xb).sum()
        k = (s * np.diag(dm)).sum() / nb if nb > 0 else 1.0
    resid = xa - k * (xb @ r)
    rms = float(np.sqrt((resid * resid).sum(axis=1).mean()))
    radius = float(np.sqrt((xa * xa).sum(axis=1).mean()))
    return rms, (rms / radius if radius > 0 else 0.0)


def edge_length_stress(a, b, links):
    """Relative edge-length stress of layout b against layout a over `links` (flat s,t pairs)."""
    pa, pb = _xy(a), _xy(b)
    n = pa.shape[0]
    st = np.asarray(links, dtype=np.float64).reshape(-1, 2)
    ok = np.isfinite(st).all(axis=1) & (st == np.floor(st)).all(axis=1) & (st >= 0).all(axis=1) & (st < n).all(axis=1)
    s, t = st[ok, 0].astype(np.int64), st[ok, 1].astype(np.int64)
    la = np.hypot(*(pa[s] - pa[t]).T)
    lb = np.hypot(*(pb[s] - pb[t]).T)
    good = np.isfinite(la) & np.isfinite(lb)
    la, lb = la[good], lb[good]
    den = float((la * la).sum())
    return float(np.sqrt(((la - lb) ** 2).sum() / den)) if den > 0 else 0.0


def agreement(a, b, links):
    """The full-run agreement figures of b against a, as a dict."""
    rms, rel = procrustes_rms(a, b)
    return dict(procrustes_rms=rms, procrustes_rms_relative=rel, edge_length_stress=edge_length_stress(a, b, links))

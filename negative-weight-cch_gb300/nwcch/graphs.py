"""Seeded synthetic workloads with integer arc weights and negative arcs.

The reference measures on DIMACS road graphs, which are not shipped with it;
these generators stand in for them with the shapes the benchmark names:

* ``grid``      - side x side 4-neighbour grid, bidirectional arcs;
* ``delaunay``  - Delaunay triangulation of seeded uniform points in the unit
                  square;
* ``road_like`` - a sparse planar graph cut out of a Delaunay triangulation:
                  its Euclidean minimum spanning tree plus random Delaunay
                  edges up to a target arc count (a road-network stand-in).

Every arc weight is ``w(u,v) = L(u,v) + h(v) - h(u)`` with ``L >= 1`` per
undirected edge and ``h`` a seeded, Gaussian-smoothed integer height field, so
downhill arcs are negative while every directed cycle sums to the positive
sum of its ``L`` terms (the metric is conservative). Weights are int32.

A graph is a dict with the reference's flat layout (python/run_nb.py:31-65):
``n``, ``off`` (int64[n+1]), ``tgt`` (int32[m]), ``x``, ``y`` (float64[n]) and
``w`` (int32[m]), plus ``h`` (the height field) and ``L`` (int32[m], the
length part of each arc).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "grid", "delaunay", "road_like", "scaled_metrics", "random_pairs",
    "inject_negative_triangle", "csr_from_edges", "ev_energies",
]


def _smooth_field(rng: np.random.Generator, side: int, sigma: float) -> np.ndarray:
    from scipy.ndimage import gaussian_filter
    noise = rng.standard_normal((side, side))
    f = gaussian_filter(noise, sigma=sigma, mode="reflect")
    f = (f - f.min()) / max(float(f.max() - f.min()), 1e-300)
    return f  # in [0, 1]


def csr_from_edges(n: int, eu: np.ndarray, ev: np.ndarray, L: np.ndarray, h: np.ndarray):
    """Directed CSR with both orientations of every undirected edge (u, v, L).
    Arcs of a vertex are sorted by head; weight = L + h[head] - h[tail]."""
    src = np.concatenate([eu, ev]).astype(np.int64)
    dst = np.concatenate([ev, eu]).astype(np.int64)
    ll = np.concatenate([L, L]).astype(np.int64)
    order = np.lexsort((dst, src))
    src, dst, ll = src[order], dst[order], ll[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, src + 1, 1)
    np.cumsum(off, out=off)
    w = ll + h[dst] - h[src]
    if w.size and (w.max() > np.iinfo(np.int32).max or w.min() < np.iinfo(np.int32).min):
        raise ValueError("arc weight does not fit in int32")
    return off, dst.astype(np.int32), w.astype(np.int32), ll.astype(np.int32)


def grid(side: int = 64, seed: int = 0, hmax: int = 200, lmin: int = 10, lmax: int = 100,
         sigma: float = 4.0) -> dict:
    """side x side 4-neighbour grid, L ~ U{lmin..lmax} per undirected edge,
    h a smoothed integer field in [-hmax, hmax]."""
    rng = np.random.default_rng(seed)
    n = side * side
    r, c = np.divmod(np.arange(n, dtype=np.int64), side)
    f = _smooth_field(rng, side, sigma)
    h = np.rint(f.reshape(-1) * 2 * hmax - hmax).astype(np.int64)
    hor = np.nonzero(c < side - 1)[0]
    ver = np.nonzero(r < side - 1)[0]
    eu = np.concatenate([hor, ver])
    ev = np.concatenate([hor + 1, ver + side])
    L = rng.integers(lmin, lmax + 1, size=eu.size)
    off, tgt, w, ll = csr_from_edges(n, eu, ev, L, h)
    return dict(n=n, off=off, tgt=tgt, w=w, L=ll, h=h, x=c.astype(np.float64),
                y=r.astype(np.float64), kind=f"grid{side}x{side}", seed=seed)


def _height_at(rng, x, y, hmax, lattice=256, sigma=None):
    f = _smooth_field(rng, lattice, sigma if sigma is not None else lattice / 24.0)
    gx = np.clip(x, 0.0, 1.0) * (lattice - 1)
    gy = np.clip(y, 0.0, 1.0) * (lattice - 1)
    i0 = np.minimum(gx.astype(np.int64), lattice - 2)
    j0 = np.minimum(gy.astype(np.int64), lattice - 2)
    fx, fy = gx - i0, gy - j0
    v = (f[j0, i0] * (1 - fx) * (1 - fy) + f[j0, i0 + 1] * fx * (1 - fy)
         + f[j0 + 1, i0] * (1 - fx) * fy + f[j0 + 1, i0 + 1] * fx * fy)
    return np.rint(v * 2 * hmax - hmax).astype(np.int64)


def delaunay_edges(pts: np.ndarray, workers: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Undirected Delaunay edges (u < v) of a 2-D point set."""
    from .delaunay import delaunay_edges as _tiled
    return _tiled(pts, workers=workers)


def delaunay(n: int = 264_000, seed: int = 0, hmax: int = 500, scale: float = 1000.0,
             workers: int = 0) -> dict:
    """Delaunay graph of n seeded uniform points; L = round(scale*|uv|)+1."""
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    h = _height_at(rng, pts[:, 0], pts[:, 1], hmax)
    eu, ev = delaunay_edges(pts, workers=workers)
    L = np.rint(scale * np.hypot(*(pts[eu] - pts[ev]).T)).astype(np.int64) + 1
    off, tgt, w, ll = csr_from_edges(n, eu, ev, L, h)
    return dict(n=n, off=off, tgt=tgt, w=w, L=ll, h=h, x=pts[:, 0].copy(), y=pts[:, 1].copy(),
                kind=f"delaunay{n}", seed=seed)


def _emst_mask(n, eu, ev, length):
    """Kruskal over the Delaunay edges (which contain the Euclidean MST),
    ties broken by edge id; in C++ (libnwcch)."""
    from . import _lib
    eu = np.ascontiguousarray(eu, np.int64)
    ev = np.ascontiguousarray(ev, np.int64)
    length = np.ascontiguousarray(length, np.float64)
    mask = np.empty(eu.size, np.uint8)
    _lib.check(_lib.host_lib().nwcch_emst_mask(n, eu.size, _lib.ptr(eu), _lib.ptr(ev), _lib.ptr(length),
                                          _lib.ptr(mask)), "emst_mask")
    return mask.astype(bool)


def road_like(n: int = 264_000, arcs: int | None = None, seed: int = 0, hmax: int = 500,
              scale: float = 1000.0, workers: int = 0) -> dict:
    """EMST of n seeded uniform points plus random Delaunay edges up to `arcs`
    directed arcs (default 2.44 n, the degree of DIMACS road graphs)."""
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    h = _height_at(rng, pts[:, 0], pts[:, 1], hmax)
    eu, ev = delaunay_edges(pts, workers=workers)
    length = np.hypot(*(pts[eu] - pts[ev]).T)
    keep = _emst_mask(n, eu, ev, length)
    target = (arcs if arcs is not None else int(round(2.4366 * n))) // 2
    extra = target - int(keep.sum())
    if extra > 0:
        rest = np.nonzero(~keep)[0]
        pick = rng.choice(rest, size=min(extra, rest.size), replace=False)
        keep[pick] = True
    eu, ev, length = eu[keep], ev[keep], length[keep]
    L = np.rint(scale * length).astype(np.int64) + 1
    off, tgt, w, ll = csr_from_edges(n, eu, ev, L, h)
    return dict(n=n, off=off, tgt=tgt, w=w, L=ll, h=h, x=pts[:, 0].copy(), y=pts[:, 1].copy(),
                kind=f"roadlike{n}", seed=seed)


def scaled_metrics(g: dict, k: int, seed: int = 0, lo: float = 0.5, hi: float = 1.5) -> np.ndarray:
    """k metrics over one topology: metric j uses h_j = round(a_j * h) with
    a_j ~ U[lo, hi] (seeded); w_j = L + h_j(v) - h_j(u). Returns int32[k, m]."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(lo, hi, size=k)
    n, off, tgt = g["n"], g["off"], g["tgt"]
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
    out = np.empty((k, tgt.size), np.int32)
    for j in range(k):
        hj = np.rint(a[j] * g["h"]).astype(np.int64)
        out[j] = (g["L"].astype(np.int64) + hj[tgt] - hj[src]).astype(np.int32)
    return out


def ev_energies(g: dict, beta_up: float = 1.0, beta_down: float = 0.6) -> np.ndarray:
    """Electric-vehicle arc energies (the reference's EV model,
    python/graphs.py:5-18 and 50-54): the length part plus beta_up per unit
    of climb, minus beta_down per unit of descent (recuperation recovers less
    than climbing costs), with the graph's own L and height field. float64[m];
    steep descents are negative and every cycle costs energy."""
    n, off, tgt = g["n"], g["off"], g["tgt"]
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
    dz = (g["h"][tgt] - g["h"][src]).astype(np.float64)
    return g["L"].astype(np.float64) + np.where(dz > 0, beta_up, beta_down) * dz


def random_pairs(n: int, count: int, seed: int = 7) -> tuple[np.ndarray, np.ndarray]:
    """Uniform random (s, t) vertex pairs (original ids)."""
    rng = np.random.default_rng(seed)
    return (rng.integers(0, n, size=count).astype(np.int64),
            rng.integers(0, n, size=count).astype(np.int64))


def inject_negative_triangle(g: dict, seed: int = 0) -> tuple[dict, tuple[int, int, int]]:
    """Pick a directed 3-cycle u->v->w->u present in the graph and set its three
    weights so that they sum to -1. Returns the modified graph (weights copied)
    and the cycle."""
    rng = np.random.default_rng(seed)
    n, off, tgt = g["n"], g["off"], g["tgt"]
    w = g["w"].copy()
    for _ in range(100000):
        u = int(rng.integers(n))
        nu = tgt[off[u]:off[u + 1]]
        if nu.size < 2:
            continue
        for v in nu:
            nv = set(tgt[off[v]:off[v + 1]].tolist())
            for x in nu:
                if x != v and int(x) in nv:
                    # u->v, v->x, x->u all exist (arcs are bidirectional)
                    a_uv = off[u] + int(np.searchsorted(nu, v))
                    nvv = tgt[off[v]:off[v + 1]]
                    a_vx = off[v] + int(np.searchsorted(nvv, x))
                    nx = tgt[off[x]:off[x + 1]]
                    a_xu = off[x] + int(np.searchsorted(nx, u))
                    w[a_uv], w[a_vx], w[a_xu] = 0, 0, -1
                    out = dict(g)
                    out["w"] = w
                    return out, (u, int(v), int(x))
    raise RuntimeError("no triangle found")

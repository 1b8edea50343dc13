"""Exact Delaunay edges of a large 2-D point set, triangulated tile by tile.

Qhull (scipy.spatial.Delaunay) is single-threaded and takes minutes at tens of
millions of points, so large sets are split into tiles triangulated in
parallel threads (Qhull releases the GIL). A triangle of a tile's local
triangulation is kept only when

* its owner is that tile: the tile containing its circumcentre, computed from
  the vertices in a canonical (sorted-id) order so every tile agrees; and
* it is provably Delaunay for the whole set: its circumcircle, clipped to the
  bounding box, lies inside the point region the tile triangulated, so the
  local empty-circle test is a global one.

Triangles whose circumcentre is near or beyond the bounding box (slivers along
the convex hull) are owned by one extra pass over a frame of points along the
boundary, with the same proof obligation. The kept triangles are distinct
Delaunay triangles; the result is complete exactly when their number equals
2n - 2 - h (h = convex-hull vertices, points in general position). If that
count check fails, the whole set is triangulated by one Qhull call instead.
"""
from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

_DIRECT_LIMIT = 400_000     # below this, one Qhull call is fastest
_TILE_POINTS = 350_000      # target points per tile


def _qhull(pts):
    from scipy.spatial import Delaunay
    return Delaunay(pts).simplices


def _circum(P, tri):
    """Canonical circumcentres (cx, cy) and squared radii of triangles `tri`
    (global ids, each row sorted ascending)."""
    a, b, c = P[tri[:, 0]], P[tri[:, 1]], P[tri[:, 2]]
    bx, by = b[:, 0] - a[:, 0], b[:, 1] - a[:, 1]
    cx, cy = c[:, 0] - a[:, 0], c[:, 1] - a[:, 1]
    d = 2.0 * (bx * cy - by * cx)
    b2, c2 = bx * bx + by * by, cx * cx + cy * cy
    ux = (cy * b2 - by * c2) / d
    uy = (bx * c2 - cx * b2) / d
    return a[:, 0] + ux, a[:, 1] + uy, ux * ux + uy * uy


def _hull_size(P):
    """Number of convex-hull vertices. Points strictly inside the polygon of
    the extreme points in 8 directions (Akl-Toussaint) cannot be hull
    vertices, so only the rest go to Qhull."""
    from scipy.spatial import ConvexHull
    keys = [P[:, 0], P[:, 1], -P[:, 0], -P[:, 1], P[:, 0] + P[:, 1], P[:, 0] - P[:, 1],
            -P[:, 0] - P[:, 1], -P[:, 0] + P[:, 1]]
    ext = np.unique([int(np.argmax(k)) for k in keys])
    E = P[ext]
    if E.shape[0] < 3:
        return ConvexHull(P).vertices.size
    ang = np.arctan2(E[:, 1] - E[:, 1].mean(), E[:, 0] - E[:, 0].mean())
    E = E[np.argsort(ang)]
    inside = np.ones(P.shape[0], bool)
    for i in range(E.shape[0]):
        a, b = E[i], E[(i + 1) % E.shape[0]]
        cross = (b[0] - a[0]) * (P[:, 1] - a[1]) - (b[1] - a[1]) * (P[:, 0] - a[0])
        inside &= cross > 0
    cand = np.nonzero(~inside)[0]
    return ConvexHull(P[cand]).vertices.size


def _edges_from_triangles(tri: np.ndarray, n: int):
    """Unique sorted edges of a triangle list (counting sort in libnwcch)."""
    import ctypes as C

    from . import _lib
    tri = np.ascontiguousarray(tri, np.int64)
    eu, ev, ne = C.c_void_p(), C.c_void_p(), C.c_int64()
    _lib.check(_lib.host_lib().nwcch_triangle_edges(n, tri.shape[0], _lib.ptr(tri), C.byref(eu), C.byref(ev),
                                               C.byref(ne)), "triangle_edges")
    return _lib.take_buffer(eu, ne.value, np.int64), _lib.take_buffer(ev, ne.value, np.int64)


def _direct(P):
    tri = np.sort(_qhull(P), axis=1)
    return _edges_from_triangles(tri, P.shape[0])


def delaunay_edges(P: np.ndarray, workers: int = 0):
    """Undirected Delaunay edges (u < v, sorted) of points P (float64[n, 2])."""
    P = np.ascontiguousarray(P, dtype=np.float64)
    n = P.shape[0]
    if n <= _DIRECT_LIMIT:
        return _direct(P)
    workers = workers or min(32, os.cpu_count() or 1)
    gx0, gy0 = P.min(axis=0)
    gx1, gy1 = P.max(axis=0)
    W, H = gx1 - gx0, gy1 - gy0
    s = math.sqrt(W * H / n)              # mean spacing
    margin, frame, gamma = 10.0 * s, 30.0 * s, 10.0 * s
    T = max(2, int(math.ceil(math.sqrt(n / _TILE_POINTS))))
    tw, th = W / T, H / T
    # bin points into cells of about margin size for region queries
    G = max(T, int(min(W, H) / margin))
    cw, ch = W / G, H / G
    ci = np.minimum(((P[:, 0] - gx0) / cw).astype(np.int64), G - 1)
    cj = np.minimum(((P[:, 1] - gy0) / ch).astype(np.int64), G - 1)
    cell = cj * G + ci
    order = np.argsort(cell, kind="stable")
    cstart = np.searchsorted(cell[order], np.arange(G * G + 1))

    def region_points(x0, x1, y0, y1):
        i0 = max(0, int((x0 - gx0) / cw)); i1 = min(G - 1, int((x1 - gx0) / cw))
        j0 = max(0, int((y0 - gy0) / ch)); j1 = min(G - 1, int((y1 - gy0) / ch))
        parts = [order[cstart[j * G + i0]:cstart[j * G + i1 + 1]] for j in range(j0, j1 + 1)]
        idx = np.concatenate(parts)
        q = P[idx]
        keep = (q[:, 0] >= x0) & (q[:, 0] <= x1) & (q[:, 1] >= y0) & (q[:, 1] <= y1)
        return idx[keep]

    sx0, sx1, sy0, sy1 = gx0 + gamma, gx1 - gamma, gy0 + gamma, gy1 - gamma

    def tile_job(t):
        ti, tj = t % T, t // T
        x0, x1 = gx0 + ti * tw, (gx0 + (ti + 1) * tw) if ti < T - 1 else gx1
        y0, y1 = gy0 + tj * th, (gy0 + (tj + 1) * th) if tj < T - 1 else gy1
        rx0, rx1 = max(gx0, x0 - margin), min(gx1, x1 + margin)
        ry0, ry1 = max(gy0, y0 - margin), min(gy1, y1 + margin)
        idx = region_points(rx0, rx1, ry0, ry1)
        tri = np.sort(idx[_qhull(P[idx])], axis=1)
        cx, cy, r2 = _circum(P, tri)
        inner = (cx > sx0) & (cx < sx1) & (cy > sy0) & (cy < sy1)
        oi = np.clip(((cx - gx0) / tw).astype(np.int64), 0, T - 1)
        oj = np.clip(((cy - gy0) / th).astype(np.int64), 0, T - 1)
        own = inner & (oi == ti) & (oj == tj)
        r = np.sqrt(r2) * (1.0 + 1e-9) + 1e-12 * (W + H)
        # a clamped side of the region is the bounding box: nothing lies beyond it
        ok = (((rx0 <= gx0) | (cx - r > rx0)) & ((rx1 >= gx1) | (cx + r < rx1))
              & ((ry0 <= gy0) | (cy - r > ry0)) & ((ry1 >= gy1) | (cy + r < ry1)))
        return tri[own & ok]

    def frame_job():
        dist = np.minimum.reduce([P[:, 0] - gx0, gx1 - P[:, 0], P[:, 1] - gy0, gy1 - P[:, 1]])
        idx = np.nonzero(dist <= frame)[0]
        tri = np.sort(idx[_qhull(P[idx])], axis=1)
        cx, cy, r2 = _circum(P, tri)
        own = ~((cx > sx0) & (cx < sx1) & (cy > sy0) & (cy < sy1))
        r = np.sqrt(r2) * (1.0 + 1e-9) + 1e-12 * (W + H)
        # the clipped circle must stay within the frame: it may not reach the
        # inner rectangle whose points the frame pass did not see
        ix0, ix1, iy0, iy1 = gx0 + frame, gx1 - frame, gy0 + frame, gy1 - frame
        dx = np.maximum(np.maximum(ix0 - cx, 0.0), cx - ix1)
        dy = np.maximum(np.maximum(iy0 - cy, 0.0), cy - iy1)
        ok = dx * dx + dy * dy > r * r
        return tri[own & ok], _hull_size(P)

    with ThreadPoolExecutor(workers) as ex:
        futs = [ex.submit(tile_job, t) for t in range(T * T)]
        ffr = ex.submit(frame_job)
        tris = [f.result() for f in futs]
        ftri, hull = ffr.result()
    tri = np.concatenate(tris + [ftri])
    if tri.shape[0] != 2 * n - 2 - hull:
        return _direct(P)
    return _edges_from_triangles(tri, n)

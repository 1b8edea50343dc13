"""The topology arrays the device derives from first/head/parent/e_arc
(csrc/topology_build.cu) against a numpy statement of the same definitions
(the host loops they replace, and python/cch_nb.py:431-515 for the arc map):
tails, elimination-tree depths, head depths, downward lists ascending in the
tail, levels (1 + the highest lower neighbour's), original arcs per shortcut
arc ascending in id, self-loops, vertices by level and the level tables.
Exact, on the golden family, the 64x64 grid and seeded 80k graphs; and a
malformed topology is refused."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import family_case, load_golden

pytestmark = pytest.mark.gpu


def expected(n, first, head, parent, e_arc):
    first = np.asarray(first, np.int64)
    head = np.asarray(head, np.int64)
    parent = np.asarray(parent, np.int64)
    e_arc = np.asarray(e_arc, np.int64)
    mp, m = head.size, e_arc.size
    deg = np.diff(first)
    tail = np.repeat(np.arange(n), deg)
    depth = np.zeros(n, np.int64)
    for x in range(n - 1, -1, -1):  # parents have higher ranks
        if parent[x] >= 0:
            depth[x] = depth[parent[x]] + 1
    lvl = np.zeros(n, np.int64)
    for x in range(n):  # rank order: lower neighbours first
        row = head[first[x]:first[x + 1]]
        if row.size:
            lvl[row] = np.maximum(lvl[row], lvl[x] + 1)
    darc = np.argsort(head, kind="stable")
    doff = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(head, minlength=n), out=doff[1:])
    mapped = e_arc >= 0
    aeidx = np.nonzero(mapped)[0][np.argsort(e_arc[mapped], kind="stable")]
    aeoff = np.zeros(mp + 1, np.int64)
    np.cumsum(np.bincount(e_arc[mapped], minlength=mp), out=aeoff[1:])
    L = int(lvl.max()) + 1 if n else 0
    level_verts = np.argsort(lvl, kind="stable")
    level_off = np.zeros(L + 1, np.int64)
    np.cumsum(np.bincount(lvl, minlength=L), out=level_off[1:])
    level_arcs = np.zeros(L + 1, np.int64)
    np.cumsum(np.bincount(lvl, weights=deg, minlength=L).astype(np.int64), out=level_arcs[1:])
    level_tri = np.bincount(lvl[head], weights=first[tail + 1] - np.arange(mp) - 1, minlength=L).astype(np.int64)
    level_maxdeg = np.zeros(L, np.int64)
    np.maximum.at(level_maxdeg, lvl, deg)
    return dict(tail=tail, depth=depth, hdep=depth[head], doff=doff, darc=darc, level=lvl, aeoff=aeoff,
                aeidx=aeidx, loops=np.nonzero(~mapped)[0], level_verts=level_verts, level_off=level_off,
                level_arcs=level_arcs, level_tri=level_tri, level_maxdeg=level_maxdeg,
                triangles=int((deg * (deg - 1) // 2).sum()), max_depth=int(depth.max()), levels=L,
                max_row=int(deg.max()) if n else 0)


def _cases():
    from nwcch import graphs as G
    from nwcch import topology as TT
    F = load_golden("family.npz")
    for i in (0, 5, 11):
        c = family_case(F, i)
        yield f"family{i}", (int(c["n"]), c["first"], c["head"], c["parent"], c["e_arc"], c["e_up"])
    z = load_golden("grid64.npz")
    yield "grid64", (int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    z = load_golden("techniques.npz")  # a forest, with self-loops
    yield "techniques", (int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    for kind in ("road", "delaunay"):
        g = {"road": G.road_like, "delaunay": G.delaunay}[kind](80_000, seed=17)
        t = TT.build_topology(g)
        yield f"{kind}80k", (t["n"], t["first"], t["head"], t["parent"], t["e_arc"], t["e_up"])


def test_device_built_arrays_equal_their_definitions(gpu):
    from nwcch.device import DeviceTopology
    for name, (n, first, head, parent, e_arc, e_up) in _cases():
        T = DeviceTopology(n, first, head, parent, e_arc, e_up)
        want = expected(n, first, head, parent, e_arc)
        assert T.triangles == want["triangles"] and T.depth == want["max_depth"], name
        assert T.levels == want["levels"] and T.max_row == want["max_row"], name
        for key in DeviceTopology._ARRAYS:
            got = T.export(key)
            assert np.array_equal(got.astype(np.int64), np.asarray(want[key], np.int64)), (name, key)


def test_malformed_topology_is_refused(gpu):
    from nwcch import _lib
    from nwcch.device import DeviceTopology
    z = load_golden("grid64.npz")
    head = z["head"].copy()
    row = int(np.argmax(np.diff(z["first"]) >= 2))
    a = int(z["first"][row])
    head[a], head[a + 1] = head[a + 1], head[a]  # a row out of order
    with pytest.raises(_lib.NwcchError):
        DeviceTopology(int(z["n"]), z["first"], head, z["parent"], z["e_arc"], z["e_up"])
    e_arc = z["e_arc"].copy()
    e_arc[3] = int(z["first"][-1])  # past the last shortcut arc
    with pytest.raises(_lib.NwcchError):
        DeviceTopology(int(z["n"]), z["first"], z["head"], z["parent"], e_arc, z["e_up"])
    # the handle is still usable for a well-formed topology afterwards
    T = DeviceTopology(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    assert T.negative_cycle_arcs(T.customize(z["w"], "int32")) == 0

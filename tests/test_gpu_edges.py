"""Edge cases on the GPU path, each against the oracle: a single vertex, a
graph with self-loops (a negative one included), disconnected components
(unreachable pairs: no path, empty shortest path), parallel arcs, weights near
the int32 limits (int32 storage saturates and says so; int64 is exact), and
empty query and update batches."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
INF = np.iinfo(np.int64).max


def _graph(n, arcs, w):
    """CSR from (u, v) arcs in the given order (edge index = position after
    a stable sort by u)."""
    arcs = np.asarray(arcs, np.int64).reshape(-1, 2)
    w = np.asarray(w, np.int64)
    order = np.argsort(arcs[:, 0], kind="stable")
    arcs, w = arcs[order], w[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, arcs[:, 0] + 1, 1)
    np.cumsum(off, out=off)
    rng = np.random.default_rng(n)
    return dict(n=n, off=off, tgt=arcs[:, 1].astype(np.int32), w=w.astype(np.int32),
                x=rng.random(n), y=rng.random(n))


def _check(gpu, oracle, g, pairs=None, storage="int32", expect_saturated=False):
    from nwcch import topology as TT
    from nwcch.device import DeviceTopology
    top = TT.build_topology(g, leaf=4)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    if expect_saturated:
        with pytest.warns(Warning):
            m = T.customize(g["w"], storage)
        assert m.saturated
        return T, m
    m = T.customize(g["w"], storage)
    up, dn = m.to_numpy()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    assert T.negative_cycle_arcs(m) == oracle.negative_cycle_arcs(oup, odn)
    n = g["n"]
    if pairs is None:
        s, t = np.meshgrid(np.arange(n), np.arange(n))
        s, t = s.ravel(), t.ravel()
    else:
        s, t = pairs
    rs, rt = top["rank"][s], top["rank"][t]
    want = oracle.query_batch(OT, oup, odn, rs, rt)
    assert np.array_equal(T.query_batch(m, rs, rt).cpu().numpy(), want)
    if storage == "int32":
        assert np.array_equal(T.query_batch(m, rs, rt, method="plain").cpu().numpy(), want)
    dist, off, path = T.query_paths(m, rs, rt)
    dist, off, path = dist.cpu().numpy(), off.cpu().numpy(), path.cpu().numpy()
    assert np.array_equal(dist, want)
    for i in range(rs.size):
        d, p = oracle.query_path(OT, oup, odn, rs[i], rt[i])
        assert np.array_equal(path[off[i]:off[i + 1]], p)
        if d == INF:
            assert p.size == 0
    return T, m


def test_single_vertex(gpu, oracle):
    g = _graph(1, np.zeros((0, 2)), [])
    T, m = _check(gpu, oracle, g)
    assert int(T.query_batch(m, [0], [0]).cpu()[0]) == 0
    assert int(T.potential(m).cpu()[0]) == 0
    assert T.update(m, [], []) == 0


def test_self_loops_and_parallel_arcs(gpu, oracle):
    arcs = [(0, 1), (0, 1), (1, 0), (1, 2), (2, 1), (2, 2), (3, 3), (2, 3), (3, 2)]
    w = [5, 3, 4, 2, 2, 7, 1, 6, 1]
    g = _graph(4, arcs, w)
    T, m = _check(gpu, oracle, g)
    assert T.negative_loops(m) == 0
    # a negative self-loop is a negative cycle the arc scan cannot see
    k = int(np.nonzero((np.repeat(np.arange(4), np.diff(g["off"])) == 3) & (g["tgt"] == 3))[0][0])
    T.update(m, [k], [-1])
    assert T.negative_loops(m) == 1


def test_disconnected_components(gpu, oracle):
    arcs = [(0, 1), (1, 0), (1, 2), (2, 1), (3, 4), (4, 3), (5, 6)]
    w = [1, -1, 2, 3, 4, -2, 7]
    g = _graph(8, arcs, w)  # vertex 7 isolated, 5 -> 6 one way only
    _check(gpu, oracle, g)


def test_weights_near_int32_limits(gpu, oracle):
    big = np.iinfo(np.int32).max - 1
    arcs = [(0, 1), (1, 2), (2, 3), (3, 0), (1, 0), (2, 1), (3, 2), (0, 3)]
    w = [big, big, big, big, 1, 1, 1, 1]
    g = _graph(4, arcs, w)
    _check(gpu, oracle, g, storage="int64")            # exact in int64
    _check(gpu, oracle, g, storage="int32", expect_saturated=True)


def test_empty_batches(gpu, oracle):
    from nwcch import graphs as G
    g = G.grid(8, seed=1)
    T, m = _check(gpu, oracle, g, pairs=(np.zeros(0, np.int64), np.zeros(0, np.int64)))
    assert T.query_batch(m, np.zeros(0, np.int32), np.zeros(0, np.int32)).numel() == 0
    assert T.update(m, [], []) == 0

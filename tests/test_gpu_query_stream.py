"""The streaming query kernel (csrc/query_stream.cu): few queries, a CTA per
chain, each chain's rows streamed into shared memory by bulk asynchronous
copies (cp.async.bulk + mbarriers) while eight warps sweep it. Its answers
must equal the oracle's ET query (python/cch_nb.py:577-615 restated) and the
other query forms' exactly: single queries and small batches, s == t, t an
ancestor of s, pairs in different trees of a forest, metrics whose values
need 64-bit labels (the kernel leaves them to the 64-bit kernel), and metric
views of a batch whose arrays are not 16-byte aligned (the kernel is not
used for them)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _graph(kind, n, seed):
    from nwcch import graphs as G
    from nwcch import topology as TT
    g = G.grid(64, seed=seed) if kind == "grid" else {"delaunay": G.delaunay, "road": G.road_like}[kind](n, seed=seed)
    return g, TT.build_topology(g)


@pytest.mark.parametrize("kind,n", [("road", 80_000), ("delaunay", 50_000), ("grid", 4096)])
def test_stream_equals_oracle(gpu, oracle, kind, n):
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph(kind, n, seed=43)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    s, t = G.random_pairs(g["n"], 200, seed=3)
    s, t = top["rank"][s].copy(), top["rank"][t].copy()
    s[:5] = t[:5]  # s == t
    t[5:10] = top["parent"][s[5:10]].clip(0)  # t an ancestor of s
    want = oracle.query_batch(OT, oup, odn, s, t)
    m = T.customize(g["w"], "int32")
    assert tune.get(T, "query_stream_max") >= 64
    for i in range(40):  # one query per call
        assert int(T.query_batch(m, s[i:i + 1], t[i:i + 1]).cpu().numpy()[0]) == want[i], i
    for lo, hi in ((0, 7), (7, 71), (71, 135)):  # small batches (the last one: 64 queries)
        assert np.array_equal(T.query_batch(m, s[lo:hi], t[lo:hi]).cpu().numpy(), want[lo:hi]), (lo, hi)
    # the same batches through the other forms
    tune.set(T, "query_stream_max", 0)
    assert np.array_equal(T.query_batch(m, s[:64], t[:64]).cpu().numpy(), want[:64])
    assert not T.check()


@pytest.mark.parametrize("ring_kb", [12, 48, 144, 0])
def test_stream_ring_sizes(gpu, oracle, ring_kb):
    """Smaller data rings hold fewer rows per item and wrap more often (the
    producer waits for released slots far more): the answers stay the
    oracle's. 0 is the default (as large as fits, at most 192 KB)."""
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph("road", 80_000, seed=47)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    s, t = G.random_pairs(g["n"], 64, seed=9)
    s, t = top["rank"][s].copy(), top["rank"][t].copy()
    want = oracle.query_batch(OT, oup, odn, s, t)
    m = T.customize(g["w"], "int32")
    tune.set(T, "query_stream_ring_kb", ring_kb)
    assert int(np.diff(top["first"]).max()) + 8 <= ring_kb * 256 // 3 or ring_kb == 0  # the kernel takes it
    for i in range(16):
        assert int(T.query_batch(m, s[i:i + 1], t[i:i + 1]).cpu().numpy()[0]) == want[i], (ring_kb, i)
        assert T.last_query_launches() == 2  # k_qstream and the (idle) 64-bit pass
    assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want)
    assert not T.check()


def test_stream_on_a_forest_and_wide_values(gpu, oracle):
    from nwcch.device import DeviceTopology
    z = load_golden("techniques.npz")
    T = DeviceTopology(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    OT = oracle.Topo(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    oup, odn = oracle.customize(OT, z["w"])
    rng = np.random.default_rng(5)
    n = int(z["n"])
    s = rng.integers(0, n, 64)
    t = np.where(rng.random(64) < 0.5, rng.integers(0, n, 64), np.clip(s + rng.integers(-2, 3, 64), 0, n - 1))
    want = oracle.query_batch(OT, oup, odn, s, t)
    assert (want == oracle.INF).any() and (want != oracle.INF).any()
    m = T.customize(z["w"], "int32")
    assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want)
    # values outside the 32-bit label bound: the 64-bit kernel answers
    from nwcch import graphs as G
    g, top = _graph("road", 30_000, seed=5)
    w = (g["w"].astype(np.int64) * 5000).astype(np.int32)
    T2 = DeviceTopology.from_dict(top)
    OT2 = oracle.Topo.from_dict(top)
    ou2, od2 = oracle.customize(OT2, w)
    s2, t2 = G.random_pairs(g["n"], 32, seed=2)
    s2, t2 = top["rank"][s2], top["rank"][t2]
    m2 = T2.customize(w, "int32")
    assert np.array_equal(T2.query_batch(m2, s2, t2).cpu().numpy(), oracle.query_batch(OT2, ou2, od2, s2, t2))


def test_stream_on_batch_views(gpu, oracle):
    """Metric k of a metric-major batch starts k * m+ words in: unless m+ is a
    multiple of 4 its arrays are not 16-byte aligned and another form answers;
    the answers are the same either way."""
    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    g, top = _graph("delaunay", 20_000, seed=6)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    W = G.scaled_metrics(g, 3, seed=4)
    b = T.customize_batch(W)
    s, t = G.random_pairs(g["n"], 16, seed=9)
    s, t = top["rank"][s], top["rank"][t]
    for k in range(3):
        ou, od = oracle.customize(OT, W[k])
        assert np.array_equal(T.query_batch(b.metric(k), s, t).cpu().numpy(), oracle.query_batch(OT, ou, od, s, t))

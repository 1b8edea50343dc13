"""The persistent launch of the levels near the root (k_sn_chain): every
level from which no level holds a warp-kernel launch or more than
NWCCH_TUNE_SN_CHAIN_MAX_ITEMS items runs as phases of one cooperative launch
with a grid barrier between phases. Its values must equal the oracle's
(python/cch_nb.py:529-563 restated) and the launch-per-level plan's exactly,
for single metrics and metric-major batches; int64 storage keeps the
launches. A barrier wait that runs out (a test hook waits for one CTA more
than the launch has) is reported as NWCCH_ERR_TIMEOUT, and the handle stays
exact afterwards."""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graph(kind, n, seed):
    from nwcch import graphs as G
    from nwcch import topology as TT
    g = G.grid(64, seed=seed) if kind == "grid" else {"delaunay": G.delaunay, "road": G.road_like}[kind](n, seed=seed)
    return g, TT.build_topology(g)


@pytest.mark.parametrize("kind,n", [("road", 80_000), ("delaunay", 50_000), ("grid", 4096)])
def test_chain_equals_oracle_and_launches(gpu, oracle, kind, n):
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph(kind, n, seed=17)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    for items in (1536, 0, 64, 1 << 30):  # a top, none, a short top, every level without warp launches
        tune.set(T, "sn_chain_max_items", items)
        assert (T.chain_phases > 0) == (items > 0)
        up, dn = T.customize(g["w"], "int32").to_numpy()
        assert np.array_equal(up, oup) and np.array_equal(dn, odn), items
    # a metric-major batch: every metric equal to its own oracle customization
    tune.set(T, "sn_chain_max_items", 1536)
    W = G.scaled_metrics(g, 3, seed=5)
    b = T.customize_batch(W)
    for k in range(3):
        ku, kd = oracle.customize(OT, W[k])
        bu, bd = b.metric(k).to_numpy()
        assert np.array_equal(bu, ku) and np.array_equal(bd, kd), k
    # int64 storage runs the same levels as launches
    up, dn = T.customize(g["w"], "int64").to_numpy()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    assert not T.check()


def test_chain_barrier_timeout_is_reported_and_recovered(gpu, oracle):
    from nwcch import _lib
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph("delaunay", 30_000, seed=23)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    tune.set(T, "sn_chain_max_items", 1536)
    assert T.chain_phases > 1
    tune.set(T, "update_spin_limit", 20_000)
    tune.set(T, "test_barrier_extra", 1)
    t0 = time.perf_counter()
    with pytest.raises(_lib.NwcchError) as exc:
        T.customize(g["w"], "int32")
    assert exc.value.code == -6  # NWCCH_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    tune.set(T, "test_barrier_extra", 0)
    tune.set(T, "update_spin_limit", 1 << 24)
    up, dn = T.customize(g["w"], "int32").to_numpy()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)


@pytest.mark.parametrize("kind,n", [("road", 80_000), ("delaunay", 50_000)])
def test_thread_kernel_equals_oracle(gpu, oracle, kind, n):
    """Tiny supernodes of the warp-kernel levels customized by one thread
    each (k_sn_thread): values equal the oracle's and the warp kernel's, in
    int32 and int64 storage and in a metric-major batch."""
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph(kind, n, seed=29)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    tune.set(T, "sn_warp_cap", 256)
    tune.set(T, "sn_warp_min_count", 64)  # the warp levels reach well up the tree
    for cap in (32, 0, 8):
        tune.set(T, "sn_thread_cap", cap)
        for storage in ("int32", "int64"):
            up, dn = T.customize(g["w"], storage).to_numpy()
            assert np.array_equal(up, oup) and np.array_equal(dn, odn), (cap, storage)
    tune.set(T, "sn_thread_cap", 32)
    W = G.scaled_metrics(g, 2, seed=8)
    b = T.customize_batch(W)
    for k in range(2):
        ku, kd = oracle.customize(OT, W[k])
        bu, bd = b.metric(k).to_numpy()
        assert np.array_equal(bu, ku) and np.array_equal(bd, kd), k
    assert not T.check()

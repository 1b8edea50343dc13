"""Failure detection on the device without a fault: a bounded wait that runs out.

The partial update runs in one cooperative launch whose levels end at a grid
barrier; every wait there is bounded and, when the bound runs out, the kernel
records ERR_TIMEOUT and returns, so the context stays usable. The test hook
NWCCH_TUNE_TEST_BARRIER_EXTRA makes each barrier wait for one block more than
the launch has (an arrival that never comes), with a short spin limit: the
call must return NWCCH_ERR_TIMEOUT within the limit, and the handle must stay
exact afterwards (the update workspace reset, the next update equal to the
oracle's and to a fresh customization). Nothing here traps, faults or waits
without a limit.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["int32", "int64"])
def test_update_barrier_timeout_is_reported_and_recovered(gpu, oracle, storage):
    from nwcch import _lib
    from nwcch import graphs as G
    from nwcch import topology as TT
    from nwcch import tune
    from nwcch.device import DeviceTopology

    g = G.delaunay(20_000, seed=31)
    top = TT.build_topology(g)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    w = g["w"].copy()
    m = T.customize(w, storage)
    rng = np.random.default_rng(3)
    idx = rng.choice(w.size, size=50, replace=False)
    val = (w[idx] + rng.integers(1, 100, size=idx.size)).astype(np.int32)

    tune.set(T, "update_small_arcs", 0)  # the grid sweep from the first level (its barriers are the test)
    tune.set(T, "update_spin_limit", 20_000)  # about 2 ms of 100 ns sleeps per wait
    tune.set(T, "test_barrier_extra", 1)
    t0 = time.perf_counter()
    with pytest.raises(_lib.NwcchError) as exc:
        T.update(m, idx, val)
    assert exc.value.code == -6  # NWCCH_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    # the context is usable and the call left w updated (its first step)
    w[idx] = val
    assert np.array_equal(m.w.cpu().numpy(), w)

    # recovery: the hook off, the metric customized again from the new
    # weights, then an ordinary update on the same handle and workspace
    tune.set(T, "test_barrier_extra", 0)
    tune.set(T, "update_spin_limit", 1 << 24)
    T.customize(m.w, storage, out=m)
    oup, odn = oracle.customize(OT, w)
    idx2 = rng.choice(w.size, size=100, replace=False)
    val2 = (w[idx2] + rng.integers(1, 100, size=idx2.size)).astype(np.int32)
    ev = T.update(m, idx2, val2)
    oev, och, _ = oracle.update(OT, w, oup, odn, idx2, val2)
    assert ev == oev
    assert np.array_equal(np.sort(m.last_changed.cpu().numpy().astype(np.int64)), np.sort(och))
    up, dn = m.to_numpy()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    fu, fd = T.customize(m.w, storage).to_numpy()
    assert np.array_equal(fu, up) and np.array_equal(fd, dn)

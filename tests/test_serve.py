"""Serving loop: continuous batching over several resident metrics with
interleaved update batches. Every answer in the mix equals the answer of the
same query alone on the same metric version, and the oracle's."""
from __future__ import annotations

import numpy as np
import pytest


def _setup(n=20_000, metrics=4, seed=5):
    from nwcch import graphs as G
    from nwcch import topology as TT
    from nwcch.device import DeviceTopology
    g = G.delaunay(n, seed=seed)
    top = TT.build_topology(g)
    T = DeviceTopology.from_dict(top)
    W = G.scaled_metrics(g, metrics, seed=2)
    return g, top, T, W


def _versions(res, W):
    """(metric index, version) -> weights after that many updates."""
    out = {}
    cur = {k: W[k].astype(np.int32).copy() for k in range(len(W))}
    ver = {k: 0 for k in cur}
    for k in cur:
        out[k, 0] = cur[k].copy()
    for (tu, j, idx, val), r in zip(res.trace.updates, res.updates):
        cur[j][idx] = val.astype(np.int32)
        ver[j] += 1
        assert r.version == ver[j]
        out[j, ver[j]] = cur[j].copy()
    return out


def _check_alone(T, res, W, oracle=None, OT=None, alone=300):
    """Every answer of the mix equals the same query alone (one per call) on
    a fresh customization of the same metric version, and the oracle's."""
    versions = _versions(res, W)
    tr = res.trace
    groups = {}
    for i in range(tr.queries):
        groups.setdefault((int(tr.q_metric[i]), int(res.version[i])), []).append(i)
    checked = 0
    for (j, v), ids in groups.items():
        ids = np.array(ids)
        m = T.customize(versions[j, v], "int32")
        s, t, got = tr.q_s[ids], tr.q_t[ids], res.result[ids]
        assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), got)
        for i in range(min(ids.size, max(0, alone - checked))):
            assert int(T.query_batch(m, s[i:i + 1], t[i:i + 1]).cpu().numpy()[0]) == got[i]
        checked += min(ids.size, alone)
        if oracle is not None:
            oup, odn = oracle.customize(OT, versions[j, v])
            assert np.array_equal(oracle.query_batch(OT, oup, odn, s[:50], t[:50]), got[:50])
    return len(groups)


def test_poisson_trace_shape():
    """Host-side trace generation: sorted arrivals, rate, conservative
    update values relative to the advancing weights."""
    from nwcch.serve import poisson_trace

    class Topo:
        n, m = 1000, 5000
    rng = np.random.default_rng(0)
    L = rng.integers(10, 100, Topo.m)
    W = {0: L.astype(np.int32).copy(), 1: (2 * L).astype(np.int32).copy()}
    w0 = {k: v.copy() for k, v in W.items()}
    tr = poisson_trace(Topo, [0, 1], rate=10_000, duration=0.5, update_every=0.05, update_sizes=(1, 7),
                       weights=W, L=L, seed=1)
    assert abs(tr.queries - 5000) < 400
    assert np.all(np.diff(tr.q_time) >= 0) and tr.q_time.max() < 0.5
    assert tr.q_s.max() < Topo.n and set(np.unique(tr.q_metric)) == {0, 1}
    assert len(tr.updates) > 0 and all(len(u[2]) in (1, 7) for u in tr.updates)
    for k in (0, 1):
        # replaying the updates on the initial weights gives the advanced
        # ones, and every arc keeps a length (weight minus height
        # difference) of at least 1
        cur = w0[k].astype(np.int64).copy()
        heights = w0[k].astype(np.int64) - L
        for _, j, idx, val in tr.updates:
            if j == k:
                cur[idx] = val
                assert np.all(cur - heights >= 1)
        assert np.array_equal(cur, W[k])


@pytest.mark.gpu
def test_serving_same_alone_and_in_mix(gpu, oracle):
    from nwcch.serve import ServingLoop, poisson_trace, run_trace, summarize
    g, top, T, W = _setup()
    OT = oracle.Topo.from_dict(top)
    keys = list(range(len(W)))
    shadow = {k: W[k].copy() for k in keys}
    trace = poisson_trace(T, keys, rate=40_000, duration=0.4, update_every=0.02, update_sizes=(1, 10, 100),
                          weights=shadow, L=g["L"], seed=3)
    assert len(trace.updates) > 5
    with ServingLoop(T, max_batch=512) as loop:
        for k in keys:
            loop.add_metric(k, W[k])
        res = run_trace(loop, trace)
        batches = loop.batches
    assert not res.errors, res.errors[:3]
    st = summarize(res)
    assert st["queries"] == trace.queries and np.all(res.version >= 0)
    assert batches < trace.queries  # queries were batched
    assert not any(r.negative_cycle for r in res.updates)
    assert _check_alone(T, res, W, oracle, OT) > len(keys)


@pytest.mark.gpu
def test_serving_admits_by_memory(gpu):
    """A budget for two resident metrics and four registered ones: metrics
    are evicted and re-admitted (customized again from their current
    weights, updates included) and every answer stays the same."""
    from nwcch.serve import ServingLoop, poisson_trace, run_trace
    g, top, T, W = _setup(n=8_000, seed=9)
    keys = list(range(len(W)))
    shadow = {k: W[k].copy() for k in keys}
    trace = poisson_trace(T, keys, rate=5_000, duration=0.4, update_every=0.05, update_sizes=(1, 50),
                          weights=shadow, L=g["L"], seed=4)
    probe = ServingLoop(T, memory_budget=1 << 40, max_batch=128)
    budget = 2 * probe.cost() + 1
    probe.close()
    with ServingLoop(T, memory_budget=budget, max_batch=128) as loop:
        for k in keys:
            loop.add_metric(k, W[k])
        res = run_trace(loop, trace)
        assert len(loop.resident()) <= 2
        assert loop.evictions > 0 and loop.admissions > len(keys)
    assert not res.errors
    _check_alone(T, res, W, alone=100)


@pytest.mark.gpu
def test_serving_plain_method_agrees(gpu):
    from nwcch.serve import ServingLoop, poisson_trace, run_trace
    g, top, T, W = _setup(n=8_000, metrics=2, seed=11)
    trace = poisson_trace(T, [0, 1], rate=10_000, duration=0.2, seed=6)
    res = {}
    for method in ("supernodal", "plain"):
        with ServingLoop(T, max_batch=256, method=method) as loop:
            for k in (0, 1):
                loop.add_metric(k, W[k])
            res[method] = run_trace(loop, trace).result
    assert np.array_equal(res["supernodal"], res["plain"])

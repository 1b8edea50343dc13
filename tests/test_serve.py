"""Serving loop: continuous batching over several resident metrics with
interleaved update batches. Every answer in the mix equals the answer of the
same query alone on the same metric version, and the oracle's."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(n=20_000, metrics=4, seed=5):
    from nwcch import graphs as G
    from nwcch import topology as TT
    from nwcch.device import DeviceTopology
    g = G.delaunay(n, seed=seed)
    top = TT.build_topology(g)
    T = DeviceTopology.from_dict(top)
    W = G.scaled_metrics(g, metrics, seed=2)
    return g, top, T, W


def _versions(reqs, W):
    """(key, version) -> weights after that many updates of the key."""
    out = {}
    cur = {k: W[k].astype(np.int32).copy() for k in range(len(W))}
    ver = {k: 0 for k in cur}
    for k in cur:
        out[k, 0] = cur[k].copy()
    for r in reqs:
        if r.kind == "update":
            cur[r.key][r.edge_idx] = r.new_w.astype(np.int32)
            ver[r.key] += 1
            assert r.version == ver[r.key]
            out[r.key, ver[r.key]] = cur[r.key].copy()
    return out


def _check_alone(T, reqs, W, oracle=None, OT=None, alone=300):
    versions = _versions(reqs, W)
    groups = {}
    for r in reqs:
        if r.kind == "query":
            groups.setdefault((r.key, r.version), []).append(r)
    checked = 0
    for (key, v), rs in groups.items():
        m = T.customize(versions[key, v], "int32")
        s = np.array([r.s for r in rs], np.int32)
        t = np.array([r.t for r in rs], np.int32)
        got = np.array([r.result for r in rs], np.int64)
        # the whole group as one batch, then single queries one per call
        assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), got)
        for i in range(min(len(rs), max(0, alone - checked))):
            assert int(T.query_batch(m, s[i:i + 1], t[i:i + 1]).cpu().numpy()[0]) == got[i]
        checked += min(len(rs), alone)
        if oracle is not None:
            oup, odn = oracle.customize(OT, versions[key, v])
            assert np.array_equal(oracle.query_batch(OT, oup, odn, s[:50], t[:50]), got[:50])
    return len(groups)


def test_serving_same_alone_and_in_mix(gpu, oracle):
    from nwcch.serve import ServingLoop, poisson_trace, summarize
    g, top, T, W = _setup()
    OT = oracle.Topo.from_dict(top)
    keys = list(range(len(W)))
    shadow = {k: W[k].copy() for k in keys}
    trace = poisson_trace(T, keys, rate=40_000, duration=0.4, update_every=0.02, update_sizes=(1, 10, 100),
                          weights=shadow, L=g["L"], seed=3)
    assert sum(r.kind == "update" for _, r in trace) > 5
    with ServingLoop(T, max_batch=512) as loop:
        for k in keys:
            loop.add_metric(k, W[k])
        reqs = loop.run_trace(trace)
        batches = loop.batches
    assert all(r.error is None for r in reqs), [r.error for r in reqs if r.error][:3]
    st = summarize(reqs)
    assert st["queries"] == sum(r.kind == "query" for _, r in trace)
    assert batches < st["queries"]  # queries were batched
    assert not any(r.negative_cycle for r in reqs if r.kind == "update")
    assert _check_alone(T, reqs, W, oracle, OT) > len(keys)


def test_serving_admits_by_memory(gpu):
    """A budget for two resident metrics and four registered ones: metrics
    are evicted and re-admitted (customized again from their current
    weights, updates included) and every answer stays the same."""
    from nwcch.serve import ServingLoop, poisson_trace
    g, top, T, W = _setup(n=8_000, seed=9)
    keys = list(range(len(W)))
    shadow = {k: W[k].copy() for k in keys}
    trace = poisson_trace(T, keys, rate=5_000, duration=0.4, update_every=0.05, update_sizes=(1, 50),
                          weights=shadow, L=g["L"], seed=4)
    probe = ServingLoop(T, memory_budget=1 << 40, max_batch=128)
    budget = 2 * probe._cost() + 1
    probe.close()
    with ServingLoop(T, memory_budget=budget, max_batch=128) as loop:
        for k in keys:
            loop.add_metric(k, W[k])
        reqs = loop.run_trace(trace)
        assert len(loop.resident()) <= 2
        assert loop.evictions > 0 and loop.admissions > len(keys)
    assert all(r.error is None for r in reqs)
    _check_alone(T, reqs, W, alone=100)


def test_serving_plain_method_agrees(gpu):
    from nwcch.serve import ServingLoop, poisson_trace
    g, top, T, W = _setup(n=8_000, metrics=2, seed=11)
    trace = poisson_trace(T, [0, 1], rate=10_000, duration=0.2, update_every=0, seed=6)
    res = {}
    for method in ("supernodal", "plain"):
        with ServingLoop(T, max_batch=256, method=method) as loop:
            for k in (0, 1):
                loop.add_metric(k, W[k])
            res[method] = [r.result for r in loop.run_trace(trace)]
    assert res["supernodal"] == res["plain"]

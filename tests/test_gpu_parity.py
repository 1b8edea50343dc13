"""GPU parity: the sm_103a kernels (through the C ABI) against the golden
vectors of the reference and against the pinned CPU oracle. Integer work, so
every comparison is exact."""
from __future__ import annotations

import functools

import numpy as np
import pytest

from conftest import family_case, i32_to_i64, load_golden

pytestmark = pytest.mark.gpu
INF = np.iinfo(np.int64).max


def dev_topo(z, n=None):
    from nwcch.device import DeviceTopology
    return DeviceTopology(int(n if n is not None else z["n"]), z["first"], z["head"], z["parent"], z["e_arc"],
                          z["e_up"])


def gpu_ranks(z, key):
    return z["rank"][z[key]]


@pytest.mark.parametrize("storage", ["int32", "int64"])
def test_techniques_union(gpu, storage):
    z = load_golden("techniques.npz")
    T = dev_topo(z)
    m = T.customize(z["w"], storage)
    up, dn = m.to_numpy()
    assert np.array_equal(up, i32_to_i64(z["up"])) and np.array_equal(dn, i32_to_i64(z["dn"]))
    assert T.negative_cycle_arcs(m) == 0 and not m.saturated
    d = T.query_batch(m, gpu_ranks(z, "qs"), gpu_ranks(z, "qt")).cpu().numpy()
    assert np.array_equal(d, i32_to_i64(z["ans"]))
    assert np.array_equal(d, i32_to_i64(z["truth"]))


@pytest.mark.parametrize("storage", ["int32", "int64"])
@pytest.mark.parametrize("i", range(12))
def test_family_customize_query(gpu, storage, i):
    c = family_case(load_golden("family.npz"), i)
    T = dev_topo(c)
    m = T.customize(c["w"], storage)
    up, dn = m.to_numpy()
    assert np.array_equal(up, i32_to_i64(c["up"])) and np.array_equal(dn, i32_to_i64(c["dn"]))
    d = T.query_batch(m, gpu_ranks(c, "qs"), gpu_ranks(c, "qt")).cpu().numpy()
    assert np.array_equal(d, c["ans"]) and np.array_equal(d, c["truth"])


@pytest.mark.parametrize("mode", ["auto", "dense"])
@pytest.mark.parametrize("storage", ["int32", "int64"])
@pytest.mark.parametrize("i", range(12))
def test_family_updates(gpu, storage, i, mode, monkeypatch):
    """Partial re-customization against the reference's recorded updates:
    evaluated count, changed set and values. "dense" stops the level sweep
    at once, so the update is finished by the dense form."""
    if mode != "auto":
        monkeypatch.setenv("NWCCH_UPDATE_MODE", mode)
    c = family_case(load_golden("family.npz"), i)
    T = dev_topo(c)
    m = T.customize(c["w"], storage)
    for st in c["step_list"]:
        ev = T.update(m, st["idx"], st["val"])
        assert ev == int(st["evaluated"])
        changed = np.sort(m.last_changed.cpu().numpy().astype(np.int64))
        assert np.array_equal(changed, st["changed"])
        up, dn = m.to_numpy()
        assert np.array_equal(up[st["changed"]], i32_to_i64(st["up"]))
        assert np.array_equal(dn[st["changed"]], i32_to_i64(st["dn"]))
        assert (m.stats["changed_negative"] > 0) == bool(st["created"])
        full = T.customize(m.w, storage)  # partial == full
        fu, fd = full.to_numpy()
        assert np.array_equal(fu, up) and np.array_equal(fd, dn)
    before = m.to_numpy()
    k = int(c["negcycle_edge"])
    T.update(m, [k], [int(c["negcycle_w"])])
    assert m.stats["changed_negative"] > 0 and T.negative_cycle_arcs(m) > 0
    T.update(m, [k], [int(c["negcycle_restore_w"])])
    assert T.negative_cycle_arcs(m) == 0
    after = m.to_numpy()
    assert np.array_equal(after[0], before[0]) and np.array_equal(after[1], before[1])
    assert np.array_equal(after[0], i32_to_i64(c["final_up"]))


def test_grid64(gpu):
    z = load_golden("grid64.npz")
    T = dev_topo(z)
    for storage in ("int32", "int64"):
        m = T.customize(z["w"], storage)
        up, dn = m.to_numpy()
        assert np.array_equal(up, i32_to_i64(z["up"])) and np.array_equal(dn, i32_to_i64(z["dn"]))
        assert T.negative_cycle_arcs(m) == int(z["neg"])
        d = T.query_batch(m, gpu_ranks(z, "qs"), gpu_ranks(z, "qt")).cpu().numpy()
        assert np.array_equal(d, z["ans"])


@pytest.mark.parametrize("name", ["grid64.npz", "delaunay_negcycle.npz"])
def test_plain_form_equals_supernodal(gpu, name):
    z = load_golden(name)
    T = dev_topo(z)
    w = z["w"] if "w" in z else z["w0"]
    a = T.customize(w, "int32", method="plain").to_numpy()
    b = T.customize(w, "int32").to_numpy()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_delaunay_negative_cycles(gpu):
    z = load_golden("delaunay_negcycle.npz")
    T = dev_topo(z)
    m = T.customize(z["w0"], "int32")
    up, dn = m.to_numpy()
    assert np.array_equal(up, i32_to_i64(z["up0"])) and np.array_equal(dn, i32_to_i64(z["dn0"]))
    assert T.negative_cycle_arcs(m) == 0
    d = T.query_batch(m, gpu_ranks(z, "qs"), gpu_ranks(z, "qt")).cpu().numpy()
    assert np.array_equal(d, z["ans0"])
    m = T.customize(z["mild_w"], "int32")
    up, dn = m.to_numpy()
    assert not m.saturated
    assert np.array_equal(up, i32_to_i64(z["mild_up"])) and np.array_equal(dn, i32_to_i64(z["mild_dn"]))
    assert T.negative_cycle_arcs(m) == int(z["mild_neg"])
    for storage in ("int32", "int64"):
        with pytest.warns(Warning):
            m = T.customize(z["wild_w"], storage)
        assert m.saturated and T.negative_cycle_arcs(m) > 0


@pytest.mark.parametrize("kind,n", [("delaunay", 40_000), ("road", 60_000)])
def test_query_forms_agree(gpu, oracle, kind, n):
    """Batched (supernodal, sync and enqueue-only) and plain queries give the
    oracle's distances, with int32 and int64 storage."""
    from nwcch import graphs as G
    from nwcch import topology as TT
    from nwcch.device import DeviceTopology
    g = {"delaunay": G.delaunay, "road": G.road_like}[kind](n, seed=33)
    top = TT.build_topology(g)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    s, t = G.random_pairs(g["n"], 4000, seed=8)
    s, t = top["rank"][s], top["rank"][t]
    s[:50] = t[:50]  # s == t as well
    want = oracle.query_batch(OT, oup, odn, s, t)
    m = T.customize(g["w"], "int32")
    assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want)
    assert np.array_equal(T.query_batch(m, s, t, method="plain").cpu().numpy(), want)
    out = T.query_batch(m, s, t, sync=False)
    gpu.cuda.synchronize()
    assert not T.check()
    assert np.array_equal(out.cpu().numpy(), want)
    m64 = T.customize(g["w"], "int64")
    assert np.array_equal(T.query_batch(m64, s, t).cpu().numpy(), want)
    # the deep-tree variant (labels in global scratch), forced
    import os
    os.environ["NWCCH_QUERY_GLOBAL_LABELS"] = "1"
    try:
        assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want)
    finally:
        del os.environ["NWCCH_QUERY_GLOBAL_LABELS"]
    # every schedule: a warp or a CTA per query, row-by-row or 32-row chunks,
    # with or without the register cap
    from nwcch import tune
    for cta_max in (0, 1 << 30):
        for rows in (1, 16, 33):
            for occ in (1, 2, 3):
                tune.set(T, "query_cta_max", cta_max)
                tune.set(T, "query_dense_rows", rows)
                tune.set(T, "query_occupancy", occ)
                assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want), (cta_max, rows, occ)
                assert np.array_equal(T.query_batch(m, s[:7], t[:7]).cpu().numpy(), want[:7])


def test_large_weights_take_the_exact_path(gpu, oracle):
    """Weights near 2^27: sums leave the +-2^28 window of the DPX fast path,
    so blocks recompute exactly; results stay equal to the oracle."""
    from nwcch import graphs as G
    from nwcch import topology as TT
    from nwcch.device import DeviceTopology
    g = G.grid(10, seed=5)
    w = (g["w"].astype(np.int64) << 20).astype(np.int32)
    top = TT.build_topology(g, leaf=8)
    T = DeviceTopology.from_dict(top)
    oup, odn = oracle.customize(oracle.Topo.from_dict(top), w)
    assert np.abs(oup[oup != INF]).max() > (1 << 28)
    for storage in ("int32", "int64"):
        m = T.customize(w, storage)
        up, dn = m.to_numpy()
        assert not m.saturated
        assert np.array_equal(up, oup) and np.array_equal(dn, odn)


@functools.lru_cache(maxsize=4)
def _seeded(kind, n, seed):
    from nwcch import graphs as G
    from nwcch import topology as TT
    g = {"delaunay": G.delaunay, "road": G.road_like}[kind](n, seed=seed)
    return g, TT.build_topology(g)


@pytest.mark.parametrize("mode", ["auto", "incremental", "dense"])
@pytest.mark.parametrize("kind,n", [("delaunay", 50_000), ("road", 80_000)])
def test_against_oracle(gpu, oracle, kind, n, mode, monkeypatch):
    if mode != "auto":
        monkeypatch.setenv("NWCCH_UPDATE_MODE", mode)
    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    g, top = _seeded(kind, n, seed=21)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    m = T.customize(g["w"], "int32")
    up, dn = m.to_numpy()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    s, t = G.random_pairs(g["n"], 3000, seed=5)
    d = T.query_batch(m, top["rank"][s], top["rank"][t]).cpu().numpy()
    assert np.array_equal(d, oracle.query_batch(OT, oup, odn, top["rank"][s], top["rank"][t]))
    # partial updates of 1, 100 and 1000 random arcs: equal to the oracle's
    # update (evaluated count, changed set, values) and to a full recompute
    rng = np.random.default_rng(9)
    w = g["w"].copy()
    for k in (1, 100, 1000):
        # raises keep the metric conservative (lowering arbitrary arcs could
        # close negative cycles, as in the reference's traffic scenario)
        idx = rng.choice(g["w"].size, size=k, replace=False)
        val = (w[idx] + rng.integers(1, 200, size=k)).astype(np.int32)
        ev = T.update(m, idx, val)
        oev, och, oneg = oracle.update(OT, w, oup, odn, idx, val)
        assert ev == oev
        assert np.array_equal(np.sort(m.last_changed.cpu().numpy().astype(np.int64)), np.sort(och))
        up, dn = m.to_numpy()
        assert np.array_equal(up, oup) and np.array_equal(dn, odn)
        assert (m.stats["changed_negative"] > 0) == (oneg > 0)
        fu, fd = T.customize(m.w, "int32").to_numpy()
        assert np.array_equal(fu, up) and np.array_equal(fd, dn)


def test_dropin_cch_nb(gpu, oracle):
    """The reference's run_nb.py call pattern, unchanged."""
    from nwcch import cch_nb as nb
    from nwcch import graphs as G
    g = G.grid(48, seed=4)
    n, off, tgt = g["n"], g["off"], g["tgt"]
    noff, nbrs, rev = nb.undirected_csr(n, off, tgt)
    rank = nb.nested_dissection(n, noff, nbrs, rev, g["x"], g["y"], 64)
    first, head, parent = nb.symbolic(n, noff, nbrs, rank)
    e_arc, e_up = nb.edge_arcs(n, off, tgt, rank, first, head)
    upw, dnw = nb.customize(n, first, head, e_arc, e_up, g["w"].astype(np.float64))
    assert nb.negative_cycle_arcs(upw, dnw) == 0
    OT = oracle.Topo(n, first, head, parent, e_arc, e_up)
    oup, odn = oracle.customize(OT, g["w"])
    ref_up, ref_dn = nb.to_reference(upw, dnw)
    assert np.array_equal(ref_up, oracle.to_float(oup)) and np.array_equal(ref_dn, oracle.to_float(odn))
    df = dr = np.full(n, np.inf)
    mark = np.zeros(n, np.int64)
    s, t = G.random_pairs(n, 50, seed=3)
    want = oracle.query_batch(OT, oup, odn, rank[s], rank[t])
    for i in range(50):
        got = nb.query(rank[s[i]], rank[t[i]], first, head, parent, upw, dnw, df, dr, mark, i + 1)
        assert got == float(want[i])


def test_cch_class_workflow(gpu, oracle):
    """python/test_cch.py's workflow on the GPU class."""
    from nwcch import graphs as G
    from nwcch.cch import CCH
    g = G.road_like(5_000, seed=8)
    c = CCH.from_graph(g)
    assert c.customize(g["w"]) == []
    assert not c.has_negative_cycle()
    rng = np.random.default_rng(1)
    for _ in range(3):
        picked = rng.choice(g["w"].size, size=10, replace=False)
        c.update_edges(list(zip(picked, g["w"][picked] + 25)))
        assert not c.update_created_negative_cycle()
        c.update_edges(list(zip(picked, g["w"][picked])))
    s, t = G.random_pairs(g["n"], 200, seed=2)
    d = c.query_batch(s, t)
    for i in range(0, 200, 40):
        bf, neg = oracle.bellman_ford(g["n"], g["off"], g["tgt"], g["w"], int(s[i]))
        want = np.inf if bf[t[i]] == INF else float(bf[t[i]])
        assert d[i] == want


def test_customize_batch(gpu, oracle):
    """K metrics in one batched launch sequence equal K single customizations
    and the oracle; per-metric scan counts; queries and partial updates on a
    metric of the batch leave the other metrics untouched."""
    from nwcch import graphs as G
    from nwcch import topology as TT
    from nwcch.device import DeviceTopology
    g = G.delaunay(30_000, seed=17)
    top = TT.build_topology(g)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    W = G.scaled_metrics(g, 6, seed=3)
    neg, _ = G.inject_negative_triangle(dict(g, w=W[4].copy()), seed=2)
    W[4] = neg["w"]
    b = T.customize_batch(W)
    assert len(b) == 6
    counts = T.negative_cycle_arcs_batch(b).cpu().numpy()
    for k in range(6):
        m = T.customize(W[k], "int32")
        up, dn = m.to_numpy()
        bu, bd = b.metric(k).to_numpy()
        assert np.array_equal(up, bu) and np.array_equal(dn, bd)
        if k != 4:  # (metric 4 has a negative cycle: its values saturate)
            oup, odn = oracle.customize(OT, W[k])
            assert np.array_equal(up, oup) and np.array_equal(dn, odn)
        assert counts[k] == T.negative_cycle_arcs(m)
        assert (counts[k] > 0) == (k == 4)
    # replay into the same buffers (captured launch graph reused)
    b2 = T.customize_batch(W, out=b)
    assert b2.up.data_ptr() == b.up.data_ptr()
    for k in (0, 5):
        assert np.array_equal(b.metric(k).to_numpy()[0], oracle.customize(OT, W[k])[0])
    s, t = G.random_pairs(g["n"], 2000, seed=4)
    s, t = top["rank"][s], top["rank"][t]
    oup, odn = oracle.customize(OT, W[1])
    assert np.array_equal(T.query_batch(b.metric(1), s, t).cpu().numpy(), oracle.query_batch(OT, oup, odn, s, t))
    before = b.up.clone(), b.dn.clone()
    rng = np.random.default_rng(1)
    idx = rng.choice(T.m, size=100, replace=False)
    w2 = W[2].copy()
    val = (w2[idx] + 50).astype(np.int32)
    T.update(b.metric(2), idx, val)
    w2[idx] = val
    fu, fd = T.customize(w2, "int32").to_numpy()
    bu, bd = b.metric(2).to_numpy()
    assert np.array_equal(fu, bu) and np.array_equal(fd, bd)
    for k in (0, 1, 3, 4, 5):
        assert gpu.equal(b.up[k], before[0][k]) and gpu.equal(b.dn[k], before[1][k])


@pytest.mark.parametrize("storage", ["int32", "int64"])
def test_potential_golden(gpu, storage):
    """The device potential equals the reference's cch_potential / CCH.potential
    (golden) on every family graph and grid64."""
    P = load_golden("potential.npz")
    F = load_golden("family.npz")
    for i in range(int(P["cases"])):
        c = family_case(F, i)
        T = dev_topo(c)
        m = T.customize(c["w"], storage)
        p = T.potential(m).cpu().numpy()[c["rank"]]
        assert np.array_equal(p, P[f"c{i}_p"])
    z = load_golden("grid64.npz")
    T = dev_topo(z)
    p = T.potential(T.customize(z["w"], storage)).cpu().numpy()[z["rank"]]
    assert np.array_equal(p, P["grid64_p"])


@pytest.mark.parametrize("kind,n", [("delaunay", 50_000), ("road", 80_000)])
def test_potential_against_oracle(gpu, oracle, kind, n):
    """Larger graphs (big supernodes take the CTA kernels): equal to the
    oracle's two sweeps and to Bellman-Ford from a virtual source; reduced
    weights w(u,v) + p(u) - p(v) are non-negative."""
    from nwcch.device import DeviceTopology
    g, top = _seeded(kind, n, seed=21)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    m = T.customize(g["w"], "int32")
    p = T.potential(m).cpu().numpy()
    assert np.array_equal(p, oracle.potential(OT, oup, odn))
    pv = p[top["rank"]]
    assert np.array_equal(pv, oracle.virtual_source_potential(g["n"], g["off"], g["tgt"], g["w"]))
    src = np.repeat(np.arange(g["n"]), np.diff(g["off"]))
    assert np.all(g["w"].astype(np.int64) + pv[src] - pv[g["tgt"]] >= 0)


@pytest.mark.parametrize("kind,n", [("delaunay", 30_000), ("road", 60_000)])
def test_query_graph_replays(gpu, oracle, kind, n):
    """Batches replayed from one captured CUDA graph give the oracle's
    distances, batch after batch (inputs copied into the graph's buffers)."""
    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    g, top = _seeded(kind, n, seed=21)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    m = T.customize(g["w"], "int32")
    qg = T.query_graph(m, 2000)
    for seed in (1, 2, 3):
        s, t = G.random_pairs(g["n"], 2000, seed=seed)
        s, t = top["rank"][s], top["rank"][t]
        d = qg.run(s, t).cpu().numpy()
        assert np.array_equal(d, oracle.query_batch(OT, oup, odn, s, t))


@pytest.mark.parametrize("kind,n", [("delaunay", 30_000), ("road", 60_000)])
def test_autotuner_keeps_answers(gpu, oracle, kind, n):
    """Every query schedule the autotuner tries gives the same answers (it
    asserts so), the chosen one equals the oracle, and an update budget is
    picked with the metric left as it was."""
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _seeded(kind, n, seed=21)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    m = T.customize(g["w"], "int32")
    s, t = G.random_pairs(g["n"], 2000, seed=12)
    s, t = top["rank"][s], top["rank"][t]
    r = tune.tune_queries(T, m, s, t, reps=1)
    # schedules, the two forms, then the top set sizes when the tile pipeline won
    tops = 5 if r["best"]["form"] == "warp" else 0
    assert len(r["trials"]) == 5 * 3 * 3 + 2 + tops
    assert tune.get(T, "query_dense_rows") == r["best"]["query_dense_rows"]
    if tops:
        assert tune.get(T, "query_top_chains") == r["best"]["query_top_chains"]
    assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), oracle.query_batch(OT, oup, odn, s, t))
    rl = tune.tune_latency(T, m, s[:6], t[:6])
    assert len(rl["trials"]) == 6
    for wide in (0, 200):  # both CTA widths on a small batch
        tune.set(T, "query_cta_wide_max", wide)
        assert np.array_equal(T.query_batch(m, s[:100], t[:100]).cpu().numpy(),
                              oracle.query_batch(OT, oup, odn, s[:100], t[:100]))
    before = m.to_numpy()
    u = tune.tune_update(T, m, sizes=(1, 20), factors=(0.5, 1.0))
    assert tune.get(T, "update_budget_ns") == u["best"]["budget_ns"]
    assert tune.get(T, "update_dense_min") == u["best"]["dense_min"] in (0, 1, 20)
    assert len(u["trials"]) == 3
    after = m.to_numpy()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    # an update at the dense threshold equals the oracle's
    tune.set(T, "update_dense_min", 5)
    w = g["w"].copy()
    idx = np.arange(0, 50) * 7
    val = (w[idx] + 3).astype(np.int32)
    ev = T.update(m, idx, val)
    oev, _, _ = oracle.update(OT, w, oup, odn, idx, val)
    up, dn = m.to_numpy()
    assert ev == oev and np.array_equal(up, oup) and np.array_equal(dn, odn)


@pytest.mark.parametrize("storage", ["int32", "int64"])
def test_query_paths_golden(gpu, storage):
    """Device paths equal the reference's CCH.query_path (golden) on every
    family graph: distances and vertex lists, ties broken the same way."""
    Pz = load_golden("paths.npz")
    F = load_golden("family.npz")
    for i in range(int(Pz["cases"])):
        c = family_case(F, i)
        T = dev_topo(c)
        m = T.customize(c["w"], storage)
        dist, off, path = T.query_paths(m, gpu_ranks(c, "qs"), gpu_ranks(c, "qt"))
        inv = np.empty_like(c["rank"])
        inv[c["rank"]] = np.arange(c["rank"].size)
        assert np.array_equal(dist.cpu().numpy(), Pz[f"c{i}_dist"])
        assert np.array_equal(off.cpu().numpy(), Pz[f"c{i}_off"])
        assert np.array_equal(inv[path.cpu().numpy()], Pz[f"c{i}_path"])


def test_query_paths_against_oracle(gpu, oracle):
    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    g, top = _seeded("road", 80_000, seed=21)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    m = T.customize(g["w"], "int32")
    s, t = G.random_pairs(g["n"], 300, seed=3)
    s, t = top["rank"][s], top["rank"][t]
    dist, off, path = T.query_paths(m, s, t, cap=16)  # too small at first: the binding retries
    dist, off, path = dist.cpu().numpy(), off.cpu().numpy(), path.cpu().numpy()
    for i in range(s.size):
        d, p = oracle.query_path(OT, oup, odn, s[i], t[i])
        assert dist[i] == d and np.array_equal(path[off[i]:off[i + 1]], p)


def test_customize_schedules_keep_values(gpu, oracle):
    """Every customization schedule the autotuner tries (which small
    supernodes one warp customizes; the plan is rebuilt each time) gives the
    oracle's values, and the chosen one stays set."""
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _seeded("road", 80_000, seed=21)
    T = DeviceTopology.from_dict(top)
    oup, odn = oracle.customize(oracle.Topo.from_dict(top), g["w"])
    r = tune.tune_customize(T, g["w"], caps=(0, 512), min_counts=(0, 4096), reps=1)
    assert len(r["trials"]) == 3 + 2 + 2 + 2  # plans, thread kernel off/on, persistent top off/on, launch forms
    assert tune.get(T, "sn_warp_cap") == r["best"]["sn_warp_cap"]
    for cap, cnt, pdl in ((512, 0, 0), (0, 0, 1), (128, 64, 1), (512, 0, 1)):
        tune.set(T, "sn_warp_cap", cap)
        tune.set(T, "sn_warp_min_count", cnt)
        tune.set(T, "pdl", pdl)
        for storage in ("int32", "int64"):
            up, dn = T.customize(g["w"], storage).to_numpy()
            assert np.array_equal(up, oup) and np.array_equal(dn, odn), (cap, cnt, pdl, storage)
        b = T.customize_batch(np.stack([g["w"], g["w"]]))
        assert np.array_equal(b.metric(1).to_numpy()[0], oup)


def test_edge_arcs_device(gpu):
    """Device arc mapping equals the host one and the reference's (golden)."""
    from nwcch import topology as TT
    F = load_golden("family.npz")
    for i in (0, 5, 11):
        c = family_case(F, i)
        ea, eu = TT.edge_arcs_device(int(c["n"]), c["off"], c["tgt"], c["rank"], c["first"], c["head"])
        assert np.array_equal(ea.cpu().numpy(), c["e_arc"]) and np.array_equal(eu.cpu().numpy(), c["e_up"])
    g, top = _seeded("road", 80_000, seed=21)
    ea, eu = TT.edge_arcs_device(g["n"], g["off"], g["tgt"], top["rank"], top["first"], top["head"])
    assert np.array_equal(ea.cpu().numpy(), top["e_arc"]) and np.array_equal(eu.cpu().numpy(), top["e_up"])


@pytest.mark.parametrize("small_arcs,small_ns,budget_ns", [
    (0, 300_000, None), (12, 300_000, None), (1 << 20, 300_000, None),
    # out of time inside a level: the one-CTA sweep hands the level over
    # part way (1 ns: before its first arc), the grid sweep stops part way
    # into the dense finish (1 ns, 20 us), or both in turn
    (1 << 20, 1, None), (0, 300_000, 1), (0, 300_000, 20_000), (1 << 20, 1, 1)])
def test_update_one_cta_sweep_and_hand_over(gpu, oracle, small_arcs, small_ns, budget_ns, monkeypatch):
    """Partial updates that sweep in one CTA, hand over to the grid sweep
    after a few evaluated arcs or part way through a level, use the grid
    sweep from the start, or stop part way through a level for the dense
    finish: the evaluated count, changed set and values equal the oracle's
    update (python/cch.py:349-402 restated) in every case."""
    if budget_ns is None:
        monkeypatch.setenv("NWCCH_UPDATE_MODE", "incremental")
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _seeded("road", 40_000, seed=33)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    m = T.customize(g["w"], "int32")
    tune.set(T, "update_small_arcs", small_arcs)
    tune.set(T, "update_small_ns", small_ns)
    if budget_ns is not None:
        tune.set(T, "update_budget_ns", budget_ns)
        tune.set(T, "update_dense_min", 0)
    rng = np.random.default_rng(17)
    w = g["w"].copy()
    for k in (1, 3, 40, 300):
        idx = rng.choice(w.size, size=k, replace=False)
        val = (w[idx] + rng.integers(1, 200, size=k)).astype(np.int32)
        ev = T.update(m, idx, val)
        oev, och, _ = oracle.update(OT, w, oup, odn, idx, val)
        assert ev == oev, (small_arcs, small_ns, budget_ns, k)
        assert np.array_equal(np.sort(m.last_changed.cpu().numpy().astype(np.int64)), np.sort(och))
        up, dn = m.to_numpy()
        assert np.array_equal(up, oup) and np.array_equal(dn, odn), (small_arcs, small_ns, budget_ns, k)

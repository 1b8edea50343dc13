"""The CPU oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py). These pin the oracle before any GPU result is
compared with it."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import battery_cases, family_case, i32_to_i64, load_golden

INF = np.iinfo(np.int64).max


def topo(oracle, z, n=None):
    return oracle.Topo(int(n if n is not None else z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])


def test_saturated_infinity_pitfall(oracle):
    # python/test_techniques.py:216-220: INF + (-5) must stay INF. Two-vertex
    # graph where vertex 1 cannot reach vertex 0 and the arc 0->1 is negative.
    T = oracle.Topo(2, [0, 1, 1], [1], [1, -1], [0], [1])
    up, dn = oracle.customize(T, np.array([-5], np.int32))
    assert up[0] == -5 and dn[0] == INF
    assert oracle.negative_cycle_arcs(up, dn) == 0
    d = oracle.query_batch(T, up, dn, [1, 0], [0, 1])
    assert d[0] == INF and d[1] == -5


def test_techniques_union(oracle):
    z = load_golden("techniques.npz")
    T = topo(oracle, z)
    up, dn = oracle.customize(T, z["w"])
    assert np.array_equal(up, i32_to_i64(z["up"]))
    assert np.array_equal(dn, i32_to_i64(z["dn"]))
    assert oracle.negative_cycle_arcs(up, dn) == 0
    ans = oracle.query_batch(T, up, dn, z["rank"][z["qs"]], z["rank"][z["qt"]])
    assert np.array_equal(ans, i32_to_i64(z["ans"]))
    # the exact ET query equals Bellman-Ford on every pair
    assert np.array_equal(ans, i32_to_i64(z["truth"]))
    assert int(z["exhaustive"]) == 14440


@pytest.mark.parametrize("i", range(12))
def test_family_customize_query(oracle, i):
    c = family_case(load_golden("family.npz"), i)
    T = topo(oracle, c)
    up, dn = oracle.customize(T, c["w"])
    assert np.array_equal(up, i32_to_i64(c["up"]))
    assert np.array_equal(dn, i32_to_i64(c["dn"]))
    ans = oracle.query_batch(T, up, dn, c["rank"][c["qs"]], c["rank"][c["qt"]])
    assert np.array_equal(ans, c["ans"])
    assert np.array_equal(ans, c["truth"])
    pup, pdn = oracle.customize_parallel(T, c["w"], threads=2)
    assert np.array_equal(pup, up) and np.array_equal(pdn, dn)


@pytest.mark.parametrize("i", [0, 4, 8, 11])
def test_family_updates(oracle, i):
    c = family_case(load_golden("family.npz"), i)
    T = topo(oracle, c)
    w = np.array(c["w"], np.int32)
    up, dn = oracle.customize(T, w)
    for st in c["step_list"]:
        ev, changed, neg = oracle.update(T, w, up, dn, st["idx"], st["val"])
        assert ev == int(st["evaluated"])
        order = np.argsort(changed)
        assert np.array_equal(changed[order], st["changed"])
        assert np.array_equal(up[st["changed"]], i32_to_i64(st["up"]))
        assert np.array_equal(dn[st["changed"]], i32_to_i64(st["dn"]))
        assert (neg > 0) == bool(st["created"])
        fup, fdn = oracle.customize(T, w)  # partial == full
        assert np.array_equal(fup, up) and np.array_equal(fdn, dn)
    # negative cycle created by an update, then removed by restoring
    before = (up.copy(), dn.copy())
    ev, changed, neg = oracle.update(T, w, up, dn, [int(c["negcycle_edge"])], [int(c["negcycle_w"])])
    assert neg > 0 and oracle.negative_cycle_arcs(up, dn) > 0
    oracle.update(T, w, up, dn, [int(c["negcycle_edge"])], [int(c["negcycle_restore_w"])])
    assert oracle.negative_cycle_arcs(up, dn) == 0
    assert np.array_equal(up, before[0]) and np.array_equal(dn, before[1])
    assert np.array_equal(up, i32_to_i64(c["final_up"])) and np.array_equal(dn, i32_to_i64(c["final_dn"]))


@pytest.mark.parametrize("i", [0, 4, 8, 11])
def test_family_updates_on_one_index(oracle, i):
    """The index built once (as the reference builds it) serves every step:
    the same counts, changed sets and values as the recorded updates."""
    c = family_case(load_golden("family.npz"), i)
    T = topo(oracle, c)
    w = np.array(c["w"], np.int32)
    up, dn = oracle.customize(T, w)
    X = oracle.UpdateIndex(T)
    for st in c["step_list"]:
        ev, changed, neg = X.update(w, up, dn, st["idx"], st["val"])
        assert ev == int(st["evaluated"])
        assert np.array_equal(np.sort(changed), st["changed"])
        assert np.array_equal(up[st["changed"]], i32_to_i64(st["up"]))
        assert np.array_equal(dn[st["changed"]], i32_to_i64(st["dn"]))
        assert (neg > 0) == bool(st["created"])
    X.update(w, up, dn, [int(c["negcycle_edge"])], [int(c["negcycle_w"])])
    X.update(w, up, dn, [int(c["negcycle_edge"])], [int(c["negcycle_restore_w"])])
    X.close()
    assert np.array_equal(up, i32_to_i64(c["final_up"])) and np.array_equal(dn, i32_to_i64(c["final_dn"]))


def test_kept_index_equals_index_per_call(oracle):
    """The kept update index (the CPU baseline of the bench's update timings)
    and the index built per call give the same counts, changed sets and
    values over a run of random raises and drops, including a change to an
    arc that the previous call changed (its queued stamp must not leak)."""
    from nwcch import graphs as G
    from nwcch import topology as TT
    g = G.road_like(6000, seed=8)
    top = TT.build_topology(g)
    T = oracle.Topo.from_dict(top)
    w1 = g["w"].astype(np.int32).copy()
    w2 = w1.copy()
    u1, d1 = oracle.customize(T, w1)
    u2, d2 = u1.copy(), d1.copy()
    X = oracle.UpdateIndex(T)
    rng = np.random.default_rng(3)
    last = None
    for step in range(12):
        k = int(rng.choice([1, 3, 20, 150]))
        idx = rng.choice(w1.size, size=k, replace=False)
        if last is not None:
            idx[0] = last
        val = (w1[idx].astype(np.int64) + rng.integers(-5, 60, size=k)).clip(1, 10**6).astype(np.int32)
        r1 = oracle.update(T, w1, u1, d1, idx, val)
        r2 = X.update(w2, u2, d2, idx, val)
        assert r1[0] == r2[0] and r1[2] == r2[2], step
        assert np.array_equal(np.sort(r1[1]), np.sort(r2[1])), step
        assert np.array_equal(u1, u2) and np.array_equal(d1, d2), step
        last = int(idx[-1])
    X.close()
    fu, fd = oracle.customize(T, w1)
    assert np.array_equal(fu, u1) and np.array_equal(fd, d1)


def test_grid64(oracle):
    z = load_golden("grid64.npz")
    T = topo(oracle, z)
    up, dn = oracle.customize(T, z["w"])
    assert np.array_equal(up, i32_to_i64(z["up"])) and np.array_equal(dn, i32_to_i64(z["dn"]))
    assert oracle.negative_cycle_arcs(up, dn) == int(z["neg"]) == 0
    ans = oracle.query_batch(T, up, dn, z["rank"][z["qs"]], z["rank"][z["qt"]], threads=2)
    assert np.array_equal(ans, z["ans"])
    pup, pdn = oracle.customize_parallel(T, z["w"], threads=4)
    assert np.array_equal(pup, up) and np.array_equal(pdn, dn)


def test_delaunay_negative_cycles(oracle):
    z = load_golden("delaunay_negcycle.npz")
    T = topo(oracle, z)
    up, dn = oracle.customize(T, z["w0"])
    assert np.array_equal(up, i32_to_i64(z["up0"])) and np.array_equal(dn, i32_to_i64(z["dn0"]))
    assert oracle.negative_cycle_arcs(up, dn) == 0
    ans = oracle.query_batch(T, up, dn, z["rank"][z["qs"]], z["rank"][z["qt"]])
    assert np.array_equal(ans, z["ans0"])
    # mild cycle: exact values; wild cycle: values explode, detection only
    up, dn = oracle.customize(T, z["mild_w"])
    assert bool(z["mild_exact"])
    assert np.array_equal(up, i32_to_i64(z["mild_up"])) and np.array_equal(dn, i32_to_i64(z["mild_dn"]))
    assert oracle.negative_cycle_arcs(up, dn) == int(z["mild_neg"])
    assert oracle.has_negative_cycle(int(z["n"]), z["off"], z["tgt"], z["mild_w"])
    assert oracle.has_negative_cycle(int(z["n"]), z["off"], z["tgt"], z["wild_w"])
    assert not oracle.has_negative_cycle(int(z["n"]), z["off"], z["tgt"], z["w0"])


def test_bellman_ford_pins_queries(oracle):
    z = load_golden("grid64.npz")
    n = int(z["n"])
    for s in range(0, n, 997):
        dist, neg = oracle.bellman_ford(n, z["off"], z["tgt"], z["w"], s)
        assert not neg
        sel = np.nonzero(z["qs"] == s)[0]
        for q in sel:
            assert dist[z["qt"][q]] == z["ans"][q]


def test_potential_against_reference(oracle):
    """cpp/cch.cpp:631-655 / python/cch.py:734-755: the oracle's two-sweep
    potential equals the reference's on every family graph and grid64, and
    the Bellman-Ford potential from a virtual source."""
    P = load_golden("potential.npz")
    F = load_golden("family.npz")
    for i in range(int(P["cases"])):
        c = family_case(F, i)
        T = topo(oracle, c)
        p = oracle.potential(T, i32_to_i64(c["up"]), i32_to_i64(c["dn"]))[c["rank"]]
        assert np.array_equal(p, P[f"c{i}_p"])
        assert np.array_equal(p, oracle.virtual_source_potential(int(c["n"]), c["off"], c["tgt"], c["w"]))
    z = load_golden("grid64.npz")
    p = oracle.potential(topo(oracle, z), i32_to_i64(z["up"]), i32_to_i64(z["dn"]))[z["rank"]]
    assert np.array_equal(p, P["grid64_p"])
    assert np.array_equal(p, oracle.virtual_source_potential(int(z["n"]), z["off"], z["tgt"], z["w"]))


def test_query_path_against_reference(oracle):
    """python/cch.py:406-507: the oracle's paths are the reference's paths
    (same choice among equal-length ones), and each realises its distance."""
    Pz = load_golden("paths.npz")
    F = load_golden("family.npz")
    for i in range(int(Pz["cases"])):
        c = family_case(F, i)
        T = topo(oracle, c)
        up, dn = i32_to_i64(c["up"]), i32_to_i64(c["dn"])
        inv = np.empty_like(c["rank"])
        inv[c["rank"]] = np.arange(c["rank"].size)
        off, path, dist = Pz[f"c{i}_off"], Pz[f"c{i}_path"], Pz[f"c{i}_dist"]
        wmap = {}
        for u in range(int(c["n"])):
            for k in range(c["off"][u], c["off"][u + 1]):
                key = (u, int(c["tgt"][k]))
                wmap[key] = min(wmap.get(key, INF), int(c["w"][k]))
        for j, (s, t) in enumerate(zip(c["qs"], c["qt"])):
            d, pr = oracle.query_path(T, up, dn, c["rank"][s], c["rank"][t])
            assert d == dist[j]
            assert np.array_equal(inv[pr], path[off[j]:off[j + 1]])
            if pr.size:
                assert sum(wmap[(int(a), int(b))] for a, b in zip(inv[pr][:-1], inv[pr][1:])) == d


def test_battery_long_profiles_against_reference(oracle):
    """battery_long.npz: profiles of up to 72 pieces (the reference's, run
    un-jitted) equal the oracle's piece for piece; answers equal too."""
    z = load_golden("battery_long.npz")
    T = oracle.Topo(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    cnt, off, pieces = oracle.battery_customize(T, z["w"], float(z["M"]))
    assert int(cnt.max()) > 32
    assert np.array_equal(cnt, z["cnt"]) and np.array_equal(off, z["poff"]) and np.array_equal(pieces, z["pieces"])
    got = oracle.battery_query_batch(T, (cnt, off, pieces), z["rank"][z["qs"]], z["rank"][z["qt"]], z["b0"])
    assert np.array_equal(got, z["ans"])
    fin = z["truth"] > -np.inf
    assert np.array_equal(got == -np.inf, ~fin)
    assert np.all(np.abs(got[fin] - z["truth"][fin]) <= 1e-6 * np.maximum(1.0, np.abs(z["truth"][fin])))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_battery_queries_match_label_correcting(oracle, seed):
    """On this project's own orders (the topologies the device path runs on),
    the oracle's battery queries equal the label-correcting search within
    the reference's tolerance, infeasible exactly when it is."""
    from nwcch import graphs as G
    from nwcch import topology as T
    g = G.delaunay(400, seed=seed)
    w = G.ev_energies(g)
    top = T.build_topology(g)
    OT = oracle.Topo.from_dict(top)
    rng = np.random.default_rng(seed)
    for M in (150.0, 600.0, 2400.0):
        prof = oracle.battery_customize(OT, w, M)
        s = rng.integers(g["n"], size=25)
        t = rng.integers(g["n"], size=25)
        b0 = rng.uniform(0, M, size=25)
        got = oracle.battery_query_batch(OT, prof, top["rank"][s], top["rank"][t], b0)
        for j in range(25):
            want = oracle.battery_label_correcting(g["n"], g["off"], g["tgt"], w, M, int(s[j]), float(b0[j]))[t[j]]
            if want == -np.inf:
                assert got[j] == -np.inf
            else:
                assert abs(got[j] - want) <= 1e-6 * max(1.0, abs(want))


def test_battery_against_reference(oracle):
    """python/cch_nb_battery.py: the oracle's profiles are the reference's
    piece for piece (same float64 operations, same merge order), its queries
    return the reference's answers exactly, and the label-correcting search
    (python/cch_nb_battery.py:316-351) the reference's too; both agree within
    the reference's own tolerance (python/run_nb_battery.py:99-104)."""
    for g, caps in battery_cases():
        T = topo(oracle, g)
        for c in caps:
            cnt, off, pieces = oracle.battery_customize(T, g["w"], float(c["M"]))
            assert np.array_equal(cnt, c["cnt"]) and np.array_equal(off, c["poff"])
            assert np.array_equal(pieces, c["pieces"])
            got = oracle.battery_query_batch(T, (cnt, off, pieces), g["rank"][c["qs"]], g["rank"][c["qt"]], c["b0"])
            assert np.array_equal(got, c["ans"])
            for j in range(c["qs"].size):
                soc = oracle.battery_label_correcting(int(g["n"]), g["off"], g["tgt"], g["w"], float(c["M"]),
                                                      int(c["qs"][j]), float(c["b0"][j]))
                want = soc[c["qt"][j]]
                assert want == c["truth"][j]
                assert (got[j] == want == -np.inf) or abs(got[j] - want) <= 1e-6 * max(1.0, abs(want))

"""Generates the golden fixtures in this directory from the REFERENCE's own code.

    python tests/golden/make_golden.py --reference <reference checkout>

Runs in a container that has the reference checkout; the fixtures it writes
travel with the repository, the reference does not. Sources of truth:

* python/cch.py (CCH: customize, query, update_edges,
  update_created_negative_cycle, has_negative_cycle), python/graphs.py,
  python/search.py and python/test_techniques.py of the reference, imported
  from the checkout;
* python/cch_nb.py, run un-jitted under a no-op `numba` stand-in;
* cpp/cch.cpp, compiled unmodified through oracle/ref_harness.cpp.

Fixtures (np.savez_compressed):

* techniques.npz  - the hand-built counterexample graphs of
  test_techniques.check_examples and every conservative 3-vertex digraph with
  weights in {-2..2} of test_techniques.check_exhaustive, as one disjoint
  union (order = vertex ids per component), with the reference's customized
  arcs and all-pairs query answers plus Bellman-Ford truths;
* family.npz      - the test_cch.run graph family (ev_grid 15, ev_geometric
  300, shifted_random 200; seeds 0-3) with weights scaled by 100 and rounded,
  the reference's order (leaf 8), customized arcs, queries, a scripted
  sequence of partial updates (raise / restore, test_cch.py:47-68) and the
  negative-cycle update scenario (test_cch.py:70-83);
* grid64.npz      - the 64x64 grid workload (4,096 vertices) with the
  reference C++ nested-dissection order, customized arcs, negative-cycle
  count and 1,000 query answers;
* delaunay_negcycle.npz - a 3,000-point Delaunay graph with one injected
  3-cycle of total weight -1: customized arcs and the scan count;
* potential.npz   - the reference's CCH potential: CCH.potential
  (python/cch.py:734-755) on every family.npz graph rebuilt in the
  reference with the fixture's order, and cch_potential (cpp/cch.cpp:631-655)
  on grid64.npz; original vertex ids;
* paths.npz       - the reference's shortest paths, CCH.query_path
  (python/cch.py:406-507), for the 50 query pairs of every family.npz graph:
  distance and vertex list (original ids), the reference's choice among
  equal-length paths;
* battery.npz     - python/cch_nb_battery.py (un-jitted) on the graphs of
  test_cch_battery.py with the reference's order: profiles for three
  capacities and 30 queries each (battery_query and battery_reference);
* battery_long.npz - the same on a 6,000-point Delaunay graph with steep
  terrain and this project's order, where profiles outgrow 32 pieces.

`--only NAME[,NAME]` regenerates some fixtures (techniques, family, grid64,
delaunay_negcycle, potential, paths, battery, battery_long); potential and
paths read family.npz (potential also grid64.npz).
"""
from __future__ import annotations

import argparse
import importlib
import itertools
import random
import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "negative-weight-cch_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

INF = float("inf")
INF32 = 0x7FFFFFFF


def import_reference(ref: Path):
    sys.path.insert(0, str(ref / "python"))
    if "numba" not in sys.modules:
        shim = types.ModuleType("numba")

        def njit(*args, **kwargs):
            if args and callable(args[0]):
                return args[0]
            return lambda f: f
        shim.njit = njit
        sys.modules["numba"] = shim
    mods = {}
    for name in ("graphs", "cch", "search", "preprocess", "test_techniques", "cch_nb"):
        mods[name] = importlib.import_module(name)
    return mods


def to_i32(a):
    """Reference float values (integral or inf) -> int32 with INF32."""
    a = np.asarray(a, dtype=np.float64)
    out = np.where(np.isinf(a), INF32, a)
    assert np.all(out == np.rint(out)) and np.all(np.abs(out[~np.isinf(a)]) < 2**31 - 1)
    return out.astype(np.int64).astype(np.int32)


def to_i64_any(a):
    """Reference float values -> int64 with INT64_MAX for inf (no range limit
    below 2^53, where the reference's doubles are exact)."""
    a = np.asarray(a, dtype=np.float64)
    fin = ~np.isinf(a)
    assert np.all(np.abs(a[fin]) < 2.0**53)
    return to_i64(a)


def to_i64(a):
    a = np.asarray(a, dtype=np.float64)
    out = np.where(np.isinf(a), np.iinfo(np.int64).max, 0).astype(np.int64)
    fin = ~np.isinf(a)
    assert np.all(a[fin] == np.rint(a[fin]))
    out[fin] = a[fin].astype(np.int64)
    return out


def adj_csr(g):
    """Directed CSR in g.adj order (= the reference's edge index order)."""
    off = np.zeros(g.n + 1, np.int64)
    for u in range(g.n):
        off[u + 1] = off[u] + len(g.adj[u])
    tgt = np.array([v for u in range(g.n) for v, _ in g.adj[u]], np.int32)
    w = np.array([w for u in range(g.n) for _, w in g.adj[u]], np.float64)
    return off, tgt, w


class Union:
    """Disjoint union of small reference CCHs, ranks contiguous per component."""

    def __init__(self):
        self.parts = []

    def add(self, c, g, pairs, answers, truths):
        off, tgt, w = adj_csr(g)
        self.parts.append(dict(n=g.n, off=off, tgt=tgt, w=w, rank=np.array(c.rank, np.int64),
                               first=np.array(c.first, np.int64), head=np.array(c.head, np.int64),
                               parent=np.array(c.parent, np.int64), e_arc=np.array(c.edge_arc, np.int64),
                               e_up=np.array(c.edge_dir, np.int8), up=np.array(c.up), dn=np.array(c.down),
                               pairs=np.array(pairs, np.int64).reshape(-1, 2), ans=np.array(answers, np.float64),
                               truth=np.array(truths, np.float64)))

    def arrays(self):
        vo = ao = mo = 0
        out = {k: [] for k in ("off", "tgt", "w", "rank", "first", "head", "parent", "e_arc", "e_up", "up", "dn",
                               "qs", "qt", "ans", "truth", "comp_v", "comp_a")}
        out["off"].append(np.zeros(1, np.int64))
        out["first"].append(np.zeros(1, np.int64))
        for p in self.parts:
            out["off"].append(p["off"][1:] + mo)
            out["tgt"].append(p["tgt"] + vo)
            out["w"].append(p["w"])
            out["rank"].append(p["rank"] + vo)
            out["first"].append(p["first"][1:] + ao)
            out["head"].append(p["head"] + vo)
            out["parent"].append(np.where(p["parent"] >= 0, p["parent"] + vo, -1))
            out["e_arc"].append(np.where(p["e_arc"] >= 0, p["e_arc"] + ao, -1))
            out["e_up"].append(p["e_up"])
            out["up"].append(p["up"])
            out["dn"].append(p["dn"])
            out["qs"].append(p["pairs"][:, 0] + vo)
            out["qt"].append(p["pairs"][:, 1] + vo)
            out["ans"].append(p["ans"])
            out["truth"].append(p["truth"])
            out["comp_v"].append([vo])
            out["comp_a"].append([ao])
            vo += p["n"]
            ao += p["first"][-1]
            mo += p["off"][-1]
        res = {k: np.concatenate([np.asarray(x) for x in v]) for k, v in out.items()}
        res["n"] = np.int64(vo)
        for k in ("w", "up", "dn", "ans", "truth"):
            res[k] = to_i32(res[k])
        for k in ("off", "tgt", "rank", "first", "head", "parent", "e_arc", "qs", "qt", "comp_v", "comp_a"):
            res[k] = res[k].astype(np.int32)
        return res


def make_techniques(R):
    tt = R["test_techniques"]
    CCH = R["cch"].CCH
    U = Union()
    recorded = []
    real_build = tt.build

    def recording_build(g, order=None, rng=None):
        c = real_build(g, order=order, rng=rng)
        if order is not None:
            recorded.append((g, c))
        return c

    tt.build = recording_build
    try:
        tt.check_examples()
    finally:
        tt.build = real_build
    seen = 0
    for g, c in recorded:
        if not c.customize(g):  # conservative examples only (as the reference asserts)
            pairs = [(s, t) for s in range(g.n) for t in range(g.n)]
            U.add(c, g, pairs, [c.query(s, t)[0] for s, t in pairs], [tt.sssp(g, s)[t] for s, t in pairs])
            seen += 1
    # test_techniques.check_exhaustive: every conservative 3-vertex digraph
    arc_pairs = [(u, v) for u in range(3) for v in range(3) if u != v]
    ex = 0
    for ws in itertools.product([None, -2, -1, 0, 1, 2], repeat=6):
        arcs = [(u, v, w) for (u, v), w in zip(arc_pairs, ws) if w is not None]
        g = tt.make_graph(3, arcs)
        if tt._has_negative_cycle(g):
            continue
        c = CCH(g, log=tt.NOLOG, order=[0, 1, 2])
        assert not c.customize(g)
        pairs = [(s, t) for s in range(3) for t in range(3)]
        D = [tt.sssp(g, s) for s in range(3)]
        U.add(c, g, pairs, [c.query(s, t)[0] for s, t in pairs], [D[s][t] for s, t in pairs])
        ex += 1
    res = U.arrays()
    res["examples"] = np.int64(seen)
    res["exhaustive"] = np.int64(ex)
    np.savez_compressed(HERE / "techniques.npz", **res)
    print(f"techniques.npz: {seen} counterexample graphs, {ex} exhaustive graphs, n={res['n']}")


def scaled(g, graphs_mod, scale=100):
    h = graphs_mod.Graph(g.n)
    for u in range(g.n):
        for v, w in g.adj[u]:
            h.add_edge(u, v, float(round(w * scale)))
    h.coords = g.coords
    return h


def make_family(R):
    gm, CCH = R["graphs"], R["cch"].CCH
    bf = R["search"].bellman_ford_query
    rng = random.Random(3)
    cases = ([("grid", gm.ev_grid(15, seed=i)) for i in range(4)]
             + [("geo", gm.ev_geometric(300, seed=i)) for i in range(4)]
             + [("shift", gm.shifted_random(200, seed=i)) for i in range(4)])
    out = {}
    for ci, (kind, g0) in enumerate(cases):
        g = scaled(g0, gm)
        xy = g.coords or [(rng.random(), rng.random()) for _ in range(g.n)]
        c = CCH(g, xy=xy, leaf=8, log=lambda *_: None)
        assert not c.customize(g), "scaled family graph has a negative cycle"
        off, tgt, w = adj_csr(g)
        pre = f"c{ci}_"
        out[pre + "n"] = np.int64(g.n)
        out[pre + "kind"] = np.array(kind)
        out[pre + "off"], out[pre + "tgt"], out[pre + "w"] = off, tgt, to_i32(w)
        out[pre + "rank"] = np.array(c.rank, np.int64)
        out[pre + "first"] = np.array(c.first, np.int64)
        out[pre + "head"] = np.array(c.head, np.int32)
        out[pre + "parent"] = np.array(c.parent, np.int64)
        out[pre + "e_arc"] = np.array(c.edge_arc, np.int64)
        out[pre + "e_up"] = np.array(c.edge_dir, np.int8)
        out[pre + "up"], out[pre + "dn"] = to_i32(c.up), to_i32(c.down)
        pairs = [(rng.randrange(g.n), rng.randrange(g.n)) for _ in range(50)]
        out[pre + "qs"] = np.array([p[0] for p in pairs], np.int64)
        out[pre + "qt"] = np.array([p[1] for p in pairs], np.int64)
        out[pre + "ans"] = to_i64([c.query(s, t)[0] for s, t in pairs])
        out[pre + "truth"] = to_i64([bf(g, s, t)[0] for s, t in pairs])
        # scripted partial updates (test_cch.py:47-68): raise 10 arcs, restore
        edges = [(u, i) for u in range(g.n) for i in range(len(g.adj[u]))]
        steps = []
        for _ in range(5):
            picked = rng.sample(range(len(edges)), 10)
            old = [g.adj[edges[k][0]][edges[k][1]][1] for k in picked]
            for weights in ([w_ + rng.randint(1, 50) * 1.0 for w_ in old], old):
                for k, w_ in zip(picked, weights):
                    u, i = edges[k]
                    g.adj[u][i] = (g.adj[u][i][0], w_)
                ev = c.update_edges(list(zip(picked, weights)))
                created = c.update_created_negative_cycle()
                ch = np.array(sorted(c.last_changed), np.int64)
                steps.append(dict(idx=np.array(picked, np.int64), val=to_i32(weights), evaluated=ev,
                                  changed=ch, up=to_i32([c.up[a] for a in ch]), dn=to_i32([c.down[a] for a in ch]),
                                  created=created))
        # negative cycle created by an update, then removed (test_cch.py:70-83)
        for k, (u, i) in enumerate(edges):
            v, w_old = g.adj[u][i]
            if any(x == u for x, _ in g.adj[v]):
                break
        # As in the reference test, a -1e6 arc closes a negative 2-cycle. The
        # customized values in its cone then grow without bound (past 2^53,
        # where the reference's doubles stop being exact), so only the
        # decisions are golden: the update reports a created cycle, and the
        # restoring update brings back every arc value exactly.
        before_up, before_dn = to_i64(c.up), to_i64(c.down)
        g.adj[u][i] = (v, -1_000_000.0)
        c.update_edges([(k, -1_000_000.0)])
        neg_created = c.update_created_negative_cycle() and c.has_negative_cycle()
        g.adj[u][i] = (v, w_old)
        c.update_edges([(k, w_old)])
        assert neg_created and not c.has_negative_cycle()
        assert np.array_equal(to_i64(c.up), before_up) and np.array_equal(to_i64(c.down), before_dn)
        out[pre + "negcycle_edge"] = np.int64(k)
        out[pre + "negcycle_w"] = np.int32(-1_000_000)
        out[pre + "negcycle_restore_w"] = np.int32(round(w_old))
        out[pre + "steps"] = np.int64(len(steps))
        for si, st in enumerate(steps):
            sp = f"{pre}s{si}_"
            for key, val in st.items():
                out[sp + key] = np.asarray(val)
        out[pre + "final_up"], out[pre + "final_dn"] = to_i32(c.up), to_i32(c.down)
    out["cases"] = np.int64(len(cases))
    np.savez_compressed(HERE / "family.npz", **out)
    print(f"family.npz: {len(cases)} graphs")


def make_grid64(R):
    from nwcch import graphs as G
    from refcpp import RefCCH
    g = G.grid(64, seed=0)
    ref = RefCCH(g)
    rank = ref.order(64)
    ref.set_order(rank)
    top = ref.symbolic()
    up, dn, _ = ref.customize(g["w"].astype(np.float64))
    neg = ref.negative_cycle_arcs(up, dn)
    # the Numba-path function of the reference gives the same arcs bit for bit
    nb = R["cch_nb"]
    up_nb, dn_nb = nb.customize(g["n"], top["first"], top["head"], top["e_arc"], top["e_up"],
                                g["w"].astype(np.float64))
    assert np.array_equal(up_nb, up) and np.array_equal(dn_nb, dn)
    s, t = G.random_pairs(g["n"], 1000, seed=7)
    ans, _ = ref.queries(up, dn, s, t)
    truth = ref.johnson_dijkstra(g["w"].astype(np.float64), s[:100], t[:100])
    assert np.array_equal(ans[:100], truth)
    np.savez_compressed(HERE / "grid64.npz", n=np.int64(g["n"]), off=g["off"], tgt=g["tgt"], w=g["w"],
                        x=g["x"], y=g["y"], rank=rank, first=top["first"], head=top["head"],
                        parent=top["parent"], e_arc=top["e_arc"], e_up=top["e_up"], up=to_i32(up),
                        dn=to_i32(dn), neg=np.int64(neg), qs=s, qt=t, ans=to_i64(ans),
                        depth=np.int64(top["depth"]), triangles=np.int64(top["triangles"]))
    print(f"grid64.npz: m+={top['first'][-1]} triangles={top['triangles']} depth={top['depth']} neg={neg}")


def make_delaunay_negcycle(R):
    """Two single -1 3-cycles injected into one Delaunay graph: one whose
    customized values stay small (exact parity expected) and one whose
    values explode past 2^53 (only the detection is golden)."""
    from nwcch import graphs as G
    from refcpp import RefCCH
    g0 = G.delaunay(3000, seed=11)
    ref = RefCCH(g0)
    rank = ref.order(64)
    ref.set_order(rank)
    top = ref.symbolic()
    up0, dn0, _ = ref.customize(g0["w"].astype(np.float64))
    assert ref.negative_cycle_arcs(up0, dn0) == 0
    s, t = G.random_pairs(g0["n"], 200, seed=7)
    ans0, _ = ref.queries(up0, dn0, s, t)
    out = dict(n=np.int64(g0["n"]), off=g0["off"], tgt=g0["tgt"], w0=g0["w"], x=g0["x"], y=g0["y"], rank=rank,
               first=top["first"], head=top["head"], parent=top["parent"], e_arc=top["e_arc"], e_up=top["e_up"],
               up0=to_i32(up0), dn0=to_i32(dn0), qs=s, qt=t, ans0=to_i64(ans0))
    for tag, seed in (("mild", 1), ("wild", 5)):
        g, cyc = G.inject_negative_triangle(g0, seed=seed)
        up, dn, _ = ref.customize(g["w"].astype(np.float64))
        neg = ref.negative_cycle_arcs(up, dn)
        assert neg > 0
        out[f"{tag}_w"] = g["w"]
        out[f"{tag}_neg"] = np.int64(neg)
        out[f"{tag}_cycle"] = np.array(cyc, np.int64)
        fin = np.concatenate([up[np.isfinite(up)], dn[np.isfinite(dn)]])
        exact = bool(np.abs(fin).max() < 2.0**31 - 1)
        out[f"{tag}_exact"] = np.bool_(exact)
        if exact:
            out[f"{tag}_up"], out[f"{tag}_dn"] = to_i32(up), to_i32(dn)
        print(f"delaunay_negcycle {tag}: neg arcs={neg} min={fin.min():.3g} exact={exact}")
    np.savez_compressed(HERE / "delaunay_negcycle.npz", **out)


def make_potential(R):
    from refcpp import RefCCH
    gm, CCH = R["graphs"], R["cch"].CCH
    fam = np.load(HERE / "family.npz")
    out = {}
    for ci in range(int(fam["cases"])):
        pre = f"c{ci}_"
        n = int(fam[pre + "n"])
        off, tgt, w = fam[pre + "off"], fam[pre + "tgt"], fam[pre + "w"]
        g = gm.Graph(n)
        for u in range(n):
            for k in range(off[u], off[u + 1]):
                g.add_edge(u, int(tgt[k]), float(w[k]))
        c = CCH(g, order=[int(r) for r in fam[pre + "rank"]], log=lambda *_: None)
        assert list(c.first) == fam[pre + "first"].tolist() and list(c.head) == fam[pre + "head"].tolist()
        assert not c.customize(g)
        assert np.array_equal(to_i32(c.up), fam[pre + "up"])
        out[pre + "p"] = to_i64(c.potential())
    z = np.load(HERE / "grid64.npz")
    ref = RefCCH(dict(n=int(z["n"]), off=z["off"], tgt=z["tgt"], x=z["x"], y=z["y"]))
    ref.set_order(z["rank"])
    ref.symbolic()
    up, dn, _ = ref.customize(z["w"].astype(np.float64))
    assert np.array_equal(to_i32(up), z["up"])
    out["grid64_p"] = to_i64(ref.cch_potential(up, dn))
    out["cases"] = fam["cases"]
    np.savez_compressed(HERE / "potential.npz", **out)
    print(f"potential.npz: {int(fam['cases'])} family graphs + grid64, min p {out['grid64_p'].min()}")


def _family_cch(R, fam, ci):
    """A family.npz graph rebuilt in the reference with the fixture's order."""
    gm, CCH = R["graphs"], R["cch"].CCH
    pre = f"c{ci}_"
    n = int(fam[pre + "n"])
    off, tgt, w = fam[pre + "off"], fam[pre + "tgt"], fam[pre + "w"]
    g = gm.Graph(n)
    for u in range(n):
        for k in range(off[u], off[u + 1]):
            g.add_edge(u, int(tgt[k]), float(w[k]))
    c = CCH(g, order=[int(r) for r in fam[pre + "rank"]], log=lambda *_: None)
    assert list(c.first) == fam[pre + "first"].tolist() and list(c.head) == fam[pre + "head"].tolist()
    assert not c.customize(g)
    return g, c


def make_paths(R):
    fam = np.load(HERE / "family.npz")
    out = {}
    for ci in range(int(fam["cases"])):
        pre = f"c{ci}_"
        g, c = _family_cch(R, fam, ci)
        dists, offs, verts = [], [0], []
        for s, t in zip(fam[pre + "qs"], fam[pre + "qt"]):
            d, path = c.query_path(int(s), int(t))
            dists.append(d)
            verts.extend(path)
            offs.append(len(verts))
            if path:  # the path realises the distance on the original graph
                assert path[0] == s and path[-1] == t
        out[pre + "dist"] = to_i64(dists)
        out[pre + "off"] = np.array(offs, np.int64)
        out[pre + "path"] = np.array(verts, np.int64)
    out["cases"] = fam["cases"]
    np.savez_compressed(HERE / "paths.npz", **out)
    print(f"paths.npz: {int(fam['cases'])} family graphs x 50 pairs")


def canonical_profiles(cnt, I1, C1, O1, pst, PI, PC, PO):
    """The reference's profile storage (inline single pieces, pooled longer
    ones; python/cch_nb_battery.py:1-8) -> cnt int32[d], off int64[d+1],
    pieces float64[total, 3] in direction order."""
    cnt = np.asarray(cnt, np.int32)
    off = np.zeros(cnt.size + 1, np.int64)
    np.cumsum(cnt, out=off[1:])
    pieces = np.empty((int(off[-1]), 3), np.float64)
    for d in range(cnt.size):
        if cnt[d] == 1:
            pieces[off[d]] = (I1[d], C1[d], O1[d])
        elif cnt[d] > 1:
            p0 = int(pst[d])
            for t in range(int(cnt[d])):
                pieces[off[d] + t] = (PI[p0 + t], PC[p0 + t], PO[p0 + t])
    return cnt, off, pieces


def make_battery(R):
    """battery.npz: python/cch_nb_battery.py, run un-jitted, on the graphs of
    python/test_cch_battery.py:54-56 (ev_grid 12 and ev_geometric 250, seeds
    0-2; float64 energies) with the reference CCH's order (leaf 8), for the
    capacities 3, 10 and 40 of test_cch_battery.py:58: the reference's
    profiles, and 30 queries per capacity (uniform s, t; b0 uniform in [0, M])
    answered by battery_query and by the label-correcting battery_reference."""
    gm, CCH = R["graphs"], R["cch"].CCH
    nbb = importlib.import_module("cch_nb_battery")
    rng = random.Random(9)
    cases = ([gm.ev_grid(12, seed=i) for i in range(3)] + [gm.ev_geometric(250, seed=i) for i in range(3)])
    out = {}
    for ci, g in enumerate(cases):
        c = CCH(g, leaf=8, log=lambda *_: None)
        off, tgt, w = adj_csr(g)
        first, head = np.array(c.first, np.int64), np.array(c.head, np.int64)
        parent, rank = np.array(c.parent, np.int64), np.array(c.rank, np.int64)
        e_arc, e_up = np.array(c.edge_arc, np.int64), np.array(c.edge_dir, np.bool_)
        pre = f"c{ci}_"
        out[pre + "n"] = np.int64(g.n)
        out[pre + "off"], out[pre + "tgt"], out[pre + "w"] = off, tgt, w
        out[pre + "rank"], out[pre + "first"], out[pre + "head"] = rank, first, head.astype(np.int32)
        out[pre + "parent"], out[pre + "e_arc"], out[pre + "e_up"] = parent, e_arc, e_up.astype(np.int8)
        soc, dsoc, mark = np.full(g.n, -np.inf), np.full(g.n, -np.inf), np.zeros(g.n, np.int64)
        q = 0
        for mi, M in enumerate((3.0, 10.0, 40.0)):
            prof = nbb.battery_customize(g.n, first, head, e_arc, e_up, w, M)
            cnt, poff, pieces = canonical_profiles(*prof)
            qs = np.array([rng.randrange(g.n) for _ in range(30)], np.int64)
            qt = np.array([rng.randrange(g.n) for _ in range(30)], np.int64)
            b0 = np.array([rng.uniform(0, M) for _ in range(30)], np.float64)
            ans, truth = [], []
            for s, t, b in zip(qs, qt, b0):
                q += 1
                ans.append(nbb.battery_query(rank[s], rank[t], b, first, head, parent, *prof, soc, dsoc, mark, q))
                truth.append(nbb.battery_reference(g.n, off, tgt, w, M, s, b)[t])
            p2 = f"{pre}m{mi}_"
            out[p2 + "M"] = np.float64(M)
            out[p2 + "cnt"], out[p2 + "poff"], out[p2 + "pieces"] = cnt, poff, pieces
            out[p2 + "qs"], out[p2 + "qt"], out[p2 + "b0"] = qs, qt, b0
            out[p2 + "ans"], out[p2 + "truth"] = np.array(ans, np.float64), np.array(truth, np.float64)
            print(f"battery case {ci} M={M}: {int(poff[-1])} pieces, largest profile {int(cnt.max())}")
    out["cases"] = np.int64(len(cases))
    out["capacities"] = np.int64(3)
    np.savez_compressed(HERE / "battery.npz", **out)
    print(f"battery.npz: {len(cases)} graphs x 3 capacities")


def make_battery_long(R):
    """battery_long.npz: python/cch_nb_battery.py, run un-jitted, on a graph
    whose profiles outgrow 32 pieces (the device keeps those in global
    memory): a 6,000-point Delaunay graph with steep terrain (this project's
    generator, heights in [-3000, 3000], EV energies) and this project's
    order; capacity 3000: the reference's profiles and 20 queries answered by
    battery_query and by battery_reference."""
    from nwcch import graphs as G
    from nwcch import topology as T
    nbb = importlib.import_module("cch_nb_battery")
    g = G.delaunay(6000, seed=5, hmax=3000)
    w = G.ev_energies(g)
    top = T.build_topology(g)
    first, head = np.asarray(top["first"], np.int64), np.asarray(top["head"], np.int64)
    parent, rank = np.asarray(top["parent"], np.int64), np.asarray(top["rank"], np.int64)
    e_arc, e_up = np.asarray(top["e_arc"], np.int64), np.asarray(top["e_up"]).astype(np.bool_)
    M = 3000.0
    prof = nbb.battery_customize(g["n"], first, head, e_arc, e_up, w, M)
    cnt, poff, pieces = canonical_profiles(*prof)
    rng = random.Random(17)
    n = int(g["n"])
    qs = np.array([rng.randrange(n) for _ in range(20)], np.int64)
    qt = np.array([rng.randrange(n) for _ in range(20)], np.int64)
    b0 = np.array([rng.uniform(0, M) for _ in range(20)], np.float64)
    soc, dsoc, mark = np.full(n, -np.inf), np.full(n, -np.inf), np.zeros(n, np.int64)
    ans, truth = [], []
    for q, (s, t, b) in enumerate(zip(qs, qt, b0)):
        ans.append(nbb.battery_query(rank[s], rank[t], b, first, head, parent, *prof, soc, dsoc, mark, q + 1))
        truth.append(nbb.battery_reference(n, g["off"], g["tgt"], w, M, s, b)[t])
    np.savez_compressed(HERE / "battery_long.npz", n=np.int64(n), off=g["off"], tgt=g["tgt"], w=w, rank=rank,
                        first=first, head=head.astype(np.int32), parent=parent, e_arc=e_arc,
                        e_up=e_up.astype(np.int8), M=np.float64(M), cnt=cnt, poff=poff, pieces=pieces, qs=qs, qt=qt,
                        b0=b0, ans=np.array(ans, np.float64), truth=np.array(truth, np.float64))
    print(f"battery_long.npz: {int(poff[-1])} pieces, largest profile {int(cnt.max())}, "
          f"{int((cnt > 32).sum())} directions above 32 pieces")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="the reference checkout")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    os.environ["NWCCH_REFERENCE_DIR"] = str(Path(args.reference).resolve())  # read by oracle/refcpp.py
    R = import_reference(Path(args.reference))
    makers = dict(techniques=make_techniques, family=make_family, grid64=make_grid64,
                  delaunay_negcycle=make_delaunay_negcycle, potential=make_potential, paths=make_paths,
                  battery=make_battery, battery_long=make_battery_long)
    only = [s for s in args.only.split(",") if s] or list(makers)
    for name in only:
        makers[name](R)


if __name__ == "__main__":
    main()

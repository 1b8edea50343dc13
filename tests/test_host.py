"""Host-side, weight-independent preprocessing (C++ in libnwcch) and the
C ABI surface. No GPU needed."""
from __future__ import annotations

import re

import numpy as np
import pytest

from conftest import ROOT, family_case, load_golden


def test_every_declared_symbol_is_exported(built_lib):
    header = (ROOT / "include" / "nwcch.h").read_text()
    names = set(re.findall(r"^\s*(?:int|void)\s+(nwcch_\w+)\s*\(", header, flags=re.M))
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(built_lib, n)]
    assert not missing, missing


def test_tuning_keys_match_the_header():
    """nwcch.tune's key names and numbers are the header's NWCCH_TUNE_*
    defines, one for one (a key added on one side only would set the wrong
    schedule or fail at run time)."""
    from nwcch import tune
    header = (ROOT / "include" / "nwcch.h").read_text()
    defined = {m.group(1).lower(): int(m.group(2))
               for m in re.finditer(r"#define NWCCH_TUNE_([A-Z0-9_]+)\s+(\d+)", header)}
    assert defined == tune.KEYS
    assert len(set(defined.values())) == len(defined)  # no number used twice
    assert tune.PLAN_KEYS <= set(defined)


def test_library_is_cuda_sm103a_build():
    import build as nwbuild
    assert "arch=compute_103a,code=sm_103a" in " ".join(nwbuild.NVCC_FLAGS)


@pytest.mark.parametrize("name", ["grid64.npz", "delaunay_negcycle.npz"])
def test_symbolic_matches_reference(built_lib, name):
    from nwcch import topology as T
    z = load_golden(name)
    g = dict(n=int(z["n"]), off=z["off"], tgt=z["tgt"])
    top = T.build_topology(g, rank=z["rank"])
    for k in ("first", "head", "parent", "e_arc", "e_up"):
        assert np.array_equal(top[k], z[k]), k


def test_symbolic_matches_reference_family(built_lib):
    from nwcch import topology as T
    F = load_golden("family.npz")
    for i in range(int(F["cases"])):
        c = family_case(F, i)
        top = T.build_topology(dict(n=int(c["n"]), off=c["off"], tgt=c["tgt"]), rank=c["rank"])
        for k in ("first", "head", "parent", "e_arc", "e_up"):
            assert np.array_equal(top[k], c[k]), (i, k)


def test_techniques_union_topology(built_lib):
    from nwcch import topology as T
    z = load_golden("techniques.npz")
    top = T.build_topology(dict(n=int(z["n"]), off=z["off"], tgt=z["tgt"]), rank=z["rank"])
    for k in ("first", "head", "parent", "e_arc", "e_up"):
        assert np.array_equal(top[k], z[k]), k


def test_nested_dissection_is_a_permutation_and_deterministic(built_lib):
    from nwcch import graphs as G
    from nwcch import topology as T
    g = G.delaunay(20_000, seed=3)
    noff, nbrs, rev = T.undirected_csr(g["n"], g["off"], g["tgt"])
    r1 = T.nested_dissection(g["n"], noff, nbrs, rev, g["x"], g["y"], 64, threads=4)
    r2 = T.nested_dissection(g["n"], noff, nbrs, rev, g["x"], g["y"], 64, threads=1)
    assert np.array_equal(np.sort(r1), np.arange(g["n"]))
    assert np.array_equal(r1, r2)  # independent of the thread schedule


def test_undirected_csr_reverse_slots(built_lib):
    from nwcch import graphs as G
    from nwcch import topology as T
    g = G.grid(16, seed=1)
    noff, nbrs, rev = T.undirected_csr(g["n"], g["off"], g["tgt"])
    owner = np.repeat(np.arange(g["n"]), np.diff(noff))
    assert np.array_equal(nbrs[rev], owner)
    assert np.array_equal(owner[rev], nbrs)


def test_triangle_edges_helper(built_lib):
    import ctypes as C

    from nwcch import _lib
    tri = np.array([[0, 1, 2], [1, 2, 3], [2, 3, 0]], np.int64)
    eu, ev, ne = C.c_void_p(), C.c_void_p(), C.c_int64()
    _lib.check(built_lib.nwcch_triangle_edges(4, 3, _lib.ptr(tri), C.byref(eu), C.byref(ev), C.byref(ne)), "tri")
    u = _lib.take_buffer(eu, ne.value, np.int64)
    v = _lib.take_buffer(ev, ne.value, np.int64)
    assert list(zip(u, v)) == [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def test_tiled_delaunay_equals_qhull():
    from nwcch import delaunay as Dl
    P = np.random.default_rng(2).random((450_000, 2))
    eu, ev = Dl.delaunay_edges(P, workers=4)
    du, dv = Dl._direct(P)
    assert np.array_equal(eu, du) and np.array_equal(ev, dv)


def test_generators_are_conservative(oracle):
    from nwcch import graphs as G
    for g in (G.grid(24, seed=2), G.delaunay(2_000, seed=2), G.road_like(3_000, seed=2)):
        assert (g["w"] < 0).any()
        assert not oracle.has_negative_cycle(g["n"], g["off"], g["tgt"], g["w"])
    g, cyc = G.inject_negative_triangle(G.delaunay(2_000, seed=4), seed=1)
    assert oracle.has_negative_cycle(g["n"], g["off"], g["tgt"], g["w"])


def test_battery_reference_layout_and_histogram():
    """nwcch.cch_nb_battery's host conversion to the reference's storage
    (inline single pieces, pooled longer profiles) keeps every profile, and
    size_histogram counts as python/cch_nb_battery.py:354-371 does."""
    from conftest import battery_cases
    from nwcch import cch_nb_battery as nbb
    for g, caps in battery_cases():
        for c in caps:
            cnt, I1, C1, O1, pst, PI, PC, PO = nbb._reference_layout(c["cnt"], c["poff"], c["pieces"])
            for d in np.nonzero(cnt)[0]:
                want = c["pieces"][c["poff"][d]:c["poff"][d + 1]]
                if cnt[d] == 1:
                    assert pst[d] == -1 and (I1[d], C1[d], O1[d]) == tuple(want[0])
                else:
                    p0 = pst[d]
                    got = np.stack([PI[p0:p0 + cnt[d]], PC[p0:p0 + cnt[d]], PO[p0:p0 + cnt[d]]], axis=1)
                    assert np.array_equal(got, want)
            assert PI.size == int(cnt[cnt > 1].sum())
            h = nbb.size_histogram(cnt)
            assert h[0] == np.count_nonzero(cnt == 0) and h[1] == np.count_nonzero(cnt == 1)
            assert h[2] == np.count_nonzero((cnt >= 2) & (cnt <= 5)) and h[7] == cnt.max()


def test_battery_energies_from_graph_objects():
    """nwcch.cch_battery reads energies in the reference's edge order from a
    Graph-like object (adjacency lists of (v, w)), a dict or an array."""
    from nwcch.cch_battery import energies_of

    class FakeGraph:
        adj = [[(1, 2.5), (2, -1.0)], [], [(0, 3.25)]]
    assert energies_of(FakeGraph()).tolist() == [2.5, -1.0, 3.25]
    assert energies_of({"w_energy": [1, 2]}).tolist() == [1.0, 2.0]
    assert energies_of(np.array([0.5])).dtype == np.float64


def test_double_order_key():
    """The integer order key the battery kernels compare doubles with
    (negative values: minus their magnitude bits; others: their bits) orders
    like IEEE comparison on every non-NaN value, -0 equal to +0."""
    rng = np.random.default_rng(4)
    vals = np.concatenate([rng.normal(0, 1e3, 4000), rng.normal(0, 1e-9, 1000),
                           np.array([0.0, -0.0, np.inf, -np.inf, 1e-308, -1e-308, 5e-324, -5e-324,
                                     1.7976931348623157e308, -1.7976931348623157e308])])
    bits = vals.view(np.int64)
    keys = np.where(bits < 0, -(bits & np.int64(0x7FFFFFFFFFFFFFFF)), bits)
    i, j = rng.integers(vals.size, size=(2, 200_000))
    assert np.array_equal(keys[i] < keys[j], vals[i] < vals[j])
    assert np.array_equal(keys[i] == keys[j], vals[i] == vals[j])


def _dominates(f, g, M, eps=1e-9):
    # python/cch_nb_battery.py:16-44
    fi, fc, fo = f
    gi, gc, go = g
    if fi > gi + eps:
        return False
    lo, hi = gi - eps, M + eps
    for b in (gi, M, fo + fc, go + gc):
        if lo <= b <= hi:
            if b < fi - eps:
                return False
            vf = min(fo, b - fc) if fo < b - fc else b - fc
            vg = min(go, b - gc) if go < b - gc else b - gc
            if vf < vg - eps:
                return False
    return True


def _merge_one(P, h, M):
    # python/cch_nb_battery.py:186-254, storage aside
    if any(_dominates(g, h, M) for g in P):
        return P
    return [g for g in P if not _dominates(h, g, M)] + [h]


def _merge_batch(P, cands, M):
    """The device's batch merge (csrc/battery.cu merge_staged), step by step:
    each candidate's first dominator in P scanning from the newest piece,
    then the in-order resolution with removal sets, then the compaction."""
    n = len(P)
    gj = []
    for h in cands:
        g = -1
        for k in range(n - 1, -1, -1):
            if _dominates(P[k], h, M):
                g = k
                break
        gj.append(g)
    removed, ins = set(), []
    for j, h in enumerate(cands):
        g = gj[j]
        if g >= 0 and g not in removed:
            continue
        d = g >= 0 and any(_dominates(P[k], h, M) for k in range(n) if k not in removed)
        d = d or any(_dominates(cands[i], h, M) for i in ins)
        if d:
            continue
        removed |= {k for k in range(n) if k not in removed and _dominates(h, P[k], M)}
        ins = [i for i in ins if not _dominates(h, cands[i], M)] + [j]
    return [P[k] for k in range(n) if k not in removed] + [cands[i] for i in ins]


def test_battery_batch_merge_equals_one_at_a_time():
    """The batch merge the battery kernel runs on 32 staged candidates gives
    the one-at-a-time merge's profile, also where the 1e-9 tolerance makes
    dominance non-transitive (pieces a fraction of the tolerance apart)."""
    rng = np.random.default_rng(12)
    M = 50.0
    jit = np.array([0.0, 0.4e-9, -0.4e-9, 0.9e-9, -0.9e-9, 1.6e-9])
    for _ in range(300):
        def piece():
            i = float(rng.integers(0, 6)) + float(rng.choice(jit))
            c = float(rng.integers(-3, 8)) + float(rng.choice(jit))
            o = min(M, float(rng.integers(5, 40)) + float(rng.choice(jit)))
            return (max(0.0, i), c, o)
        P = []
        for _ in range(int(rng.integers(0, 12))):
            P = _merge_one(P, piece(), M)
        cands = [piece() for _ in range(int(rng.integers(1, 33)))]
        want = P
        for h in cands:
            want = _merge_one(want, h, M)
        assert _merge_batch(P, cands, M) == want


def _key(x):
    b = int(np.array([x], np.float64).view(np.int64)[0])
    return -(b & 0x7FFFFFFFFFFFFFFF) if b < 0 else b


def _derive(p, M, eps=1e-9):
    """csrc/battery.cu derive(): the per-piece values of the dominance test."""
    i, c, o = p
    oc = o + c

    def mref(a, x):
        return a if _key(a) < _key(x) else x
    vM = mref(o, M - c)
    v3 = mref(o, oc - c)
    r = dict(i=i, c=c, o=o, oc=oc, ki=_key(i), kipe=_key(i + eps), kime=_key(i - eps), ko=_key(o), koc=_key(oc),
             kv0m=_key(mref(o, i - c) - eps), kvM=_key(vM), kvMm=_key(vM - eps), kom=_key(o - eps), kv3=_key(v3),
             kv3m=_key(v3 - eps))
    kM, kMpe = _key(M), _key(M + eps)
    r.update(R0=r["ki"] <= kMpe, R1=r["kime"] <= kM, R2=r["koc"] <= kMpe,
             R3=r["kime"] <= r["koc"] and r["koc"] <= kMpe, MLT=kM < r["kime"], OCLT=r["koc"] < r["kime"])
    return r


def _dominates_keys(F, G, eps=1e-9):
    """csrc/battery.cu dominates(): keys, precomputed values, skipped
    subtractions."""
    if F["ki"] > G["kipe"]:
        return False
    if G["R0"]:
        if G["ki"] < F["kime"] or F["ko"] < G["kv0m"] or _key(G["i"] - F["c"]) < G["kv0m"]:
            return False
    if G["R1"] and (F["MLT"] or F["kvM"] < G["kvMm"]):
        return False
    if F["R2"] and G["kime"] <= F["koc"]:
        if F["OCLT"]:
            return False
        if F["kv3"] < G["kom"]:
            y = F["oc"] - G["c"]
            vg = G["o"] if G["ko"] < _key(y) else y
            if F["kv3"] < _key(vg - eps):
                return False
    if G["R3"]:
        if G["koc"] < F["kime"] or F["ko"] < G["kv3m"] or _key(G["oc"] - F["c"]) < G["kv3m"]:
            return False
    return True


def test_battery_dominance_restatement():
    """The device's dominance test (order keys, per-piece values, skipped
    subtractions) answers as the reference's on random pieces, near-ties of
    a fraction of the tolerance and signed zeros included."""
    rng = np.random.default_rng(8)
    jit = [0.0, 0.3e-9, -0.3e-9, 1e-9, -1e-9, 2.2e-9]
    for M in (7.0, 40.0, 1e3):
        for _ in range(4000):
            def piece():
                i = abs(float(rng.integers(0, 9)) + float(rng.choice(jit)))
                c = float(rng.integers(-6, 10)) + float(rng.choice(jit))
                o = min(M, float(rng.integers(-2, 30)) + float(rng.choice(jit)))
                return (i, -0.0 if c == 0 and rng.random() < 0.5 else c, o)
            f, g = piece(), piece()
            assert _dominates_keys(_derive(f, M), _derive(g, M)) == _dominates(f, g, M), (f, g, M)
            # compose (python/cch_nb_battery.py:159-173) on keys, bit for bit
            want = None
            if not f[2] < g[0] - 1e-9:
                hi = f[0] if f[0] > g[0] + f[1] else g[0] + f[1]
                if not hi > M + 1e-9:
                    hc = f[1] + g[1]
                    ho = g[2]
                    if f[2] - g[1] < ho:
                        ho = f[2] - g[1]
                    if M - hc < ho:
                        ho = M - hc
                    want = (hi, hc, ho)
            got = None
            if not _key(f[2]) < _key(g[0] - 1e-9):
                s = g[0] + f[1]
                hi = f[0] if _key(f[0]) > _key(s) else s
                if not _key(hi) > _key(M + 1e-9):
                    hc = f[1] + g[1]
                    ho = g[2]
                    if _key(f[2] - g[1]) < _key(ho):
                        ho = f[2] - g[1]
                    if _key(M - hc) < _key(ho):
                        ho = M - hc
                    got = (hi, hc, ho)
            assert (got is None) == (want is None)
            if got is not None:
                assert np.array(got).view(np.int64).tolist() == np.array(want).view(np.int64).tolist()


def test_ev_energies_are_conservative(oracle):
    """The EV energies of a generated graph: steep descents are negative, and
    no cycle gains charge (label correcting from a vertex converges to a
    charge no higher than the start where the start is the capacity)."""
    from nwcch import graphs as G
    g = G.delaunay(2_000, seed=3)
    w = G.ev_energies(g)
    assert (w < 0).any() and (w > 0).any()
    soc = oracle.battery_label_correcting(g["n"], g["off"], g["tgt"], w, 1e9, 0, 1e9)
    assert soc[0] == 1e9 and np.all(soc <= 1e9)


def test_topology_create_rejects_bad_input_without_gpu(built_lib):
    """The row offsets are checked on the host before any device work (the
    rows themselves on the device: tests/test_gpu_topology_build.py)."""
    import ctypes as C

    from nwcch import _lib
    first = np.array([0, 1, 0], np.int64)  # row offsets must not decrease
    head = np.array([1], np.int32)
    parent = np.array([1, -1], np.int32)
    e_arc = np.zeros(0, np.int64)
    e_up = np.zeros(0, np.int8)
    h = C.c_void_p()
    rc = built_lib.nwcch_topology_create(2, _lib.ptr(first), _lib.ptr(head), _lib.ptr(parent), 0, _lib.ptr(e_arc),
                                         _lib.ptr(e_up), C.byref(h))
    assert rc == -4  # NWCCH_ERR_TOPOLOGY


def test_battery_entry_points_reject_null_handles_without_gpu(built_lib):
    """The battery C ABI checks its handles before any device work."""
    import ctypes as C
    L = C.CDLL(built_lib._name)  # own function objects: the package's signatures stay as registered
    L.nwcch_battery_customize.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                          C.POINTER(C.c_void_p)]
    L.nwcch_battery_info.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.nwcch_battery_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nwcch_battery_query.argtypes = [C.c_void_p] * 5 + [C.c_int64, C.c_void_p, C.c_void_p]
    L.nwcch_battery_free.argtypes = [C.c_void_p]
    L.nwcch_battery_free.restype = None
    out = C.c_void_p()
    assert L.nwcch_battery_customize(None, None, 1.0, None, C.byref(out)) == -1
    assert L.nwcch_battery_info(None, None, None) == -1
    assert L.nwcch_battery_export(None, None, None, None) == -1
    assert L.nwcch_battery_query(None, None, None, None, None, 0, None, None) == -1
    L.nwcch_battery_free(None)  # no-op

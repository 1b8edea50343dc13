"""Battery-constrained profiles on the GPU (battery.cu through the C ABI)
against the reference's own profiles and answers (battery.npz, made by
python/cch_nb_battery.py) and against the pinned CPU oracle. float64 work in
the reference's operations and order: profiles and answers are compared
exactly; the label-correcting truth within the reference's tolerance
(python/run_nb_battery.py:99-104)."""
from __future__ import annotations

import functools

import numpy as np
import pytest

from conftest import battery_cases

pytestmark = pytest.mark.gpu


def dev_topo(z):
    from nwcch.device import DeviceTopology
    return DeviceTopology(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])


def close(got, want):
    both_inf = (got == -np.inf) & (want == -np.inf)
    ok = np.abs(got - want) <= 1e-6 * np.maximum(1.0, np.abs(want))
    return bool(np.all(both_inf | ok))


def test_battery_golden(gpu):
    """Every battery.npz graph and capacity: the device profiles are the
    reference's piece for piece, the answers its answers."""
    from nwcch import battery
    for g, caps in battery_cases():
        T = dev_topo(g)
        for c in caps:
            b = battery.customize(T, g["w"], float(c["M"]))
            cnt, off, pieces = b.export()
            assert np.array_equal(cnt, c["cnt"]) and np.array_equal(off, c["poff"])
            assert np.array_equal(pieces, c["pieces"])
            assert b.pieces == int(c["poff"][-1]) and b.largest == int(c["cnt"].max())
            got = b.query(g["rank"][c["qs"]], g["rank"][c["qt"]], c["b0"]).cpu().numpy()
            assert np.array_equal(got, c["ans"])
            assert close(got, c["truth"])


def test_battery_golden_long_profiles(gpu):
    """battery_long.npz: profiles of up to 72 pieces, built partly in the
    warps' global buffers, equal to the reference's piece for piece."""
    from conftest import load_golden
    from nwcch import battery
    z = load_golden("battery_long.npz")
    T = dev_topo(z)
    b = battery.customize(T, z["w"], float(z["M"]))
    cnt, off, pieces = b.export()
    assert np.array_equal(cnt, z["cnt"]) and np.array_equal(off, z["poff"]) and np.array_equal(pieces, z["pieces"])
    got = b.query(z["rank"][z["qs"]], z["rank"][z["qt"]], z["b0"]).cpu().numpy()
    assert np.array_equal(got, z["ans"])


@functools.lru_cache(maxsize=None)
def _ev_case(n: int):
    import oracle as orc
    from nwcch import graphs as G
    from nwcch import topology as Tm
    g = G.delaunay(n, seed=1)
    w = G.ev_energies(g)
    top = Tm.build_topology(g)
    OT = orc.Topo.from_dict(top)
    rng = np.random.default_rng(21)
    big = 1e15
    ds = []
    for _ in range(12):
        s, t = (int(v) for v in rng.integers(n, size=2))
        ds.append(big - orc.battery_label_correcting(n, g["off"], g["tgt"], w, big, s, big)[t])
    return g, w, top, OT, float(np.median(ds))


@pytest.mark.parametrize("factor", [0.25, 1.0, 4.0])
def test_battery_against_oracle_delaunay(gpu, oracle, factor):
    """A 20,000-point Delaunay graph with EV energies (profiles of up to about
    40 pieces, so some outgrow the registers): profiles equal to the oracle's,
    queries equal on 400 pairs, and within tolerance of label correcting."""
    from nwcch import battery
    from nwcch.device import DeviceTopology
    g, w, top, OT, D = _ev_case(20_000)
    M = factor * D
    T = DeviceTopology.from_dict(top)
    b = battery.customize(T, w, M)
    cnt, off, pieces = b.export()
    ocnt, ooff, opieces = oracle.battery_customize(OT, w, M)
    assert np.array_equal(cnt, ocnt) and np.array_equal(off, ooff) and np.array_equal(pieces, opieces)
    assert b.largest == int(ocnt.max())
    rng = np.random.default_rng(5)
    s = rng.integers(g["n"], size=400)
    t = rng.integers(g["n"], size=400)
    b0 = rng.uniform(0, M, size=400)
    got = b.query(top["rank"][s], top["rank"][t], b0).cpu().numpy()
    want = oracle.battery_query_batch(OT, (ocnt, ooff, opieces), top["rank"][s], top["rank"][t], b0)
    assert np.array_equal(got, want)
    # small batches take the CTA-per-query form: same answers
    small = b.query(top["rank"][s[:100]], top["rank"][t[:100]], b0[:100]).cpu().numpy()
    assert np.array_equal(small, want[:100])
    truth = np.array([oracle.battery_label_correcting(g["n"], g["off"], g["tgt"], w, M, int(s[j]),
                                                      float(b0[j]))[t[j]] for j in range(20)])
    assert close(got[:20], truth)


def test_battery_regrowth(gpu):
    """A pool far too small and the smallest profile buffer: the
    customization grows them, reruns, and returns the same profiles."""
    from nwcch import battery, tune
    from nwcch.device import DeviceTopology
    g, w, top, OT, D = _ev_case(20_000)
    T = DeviceTopology.from_dict(top)
    ref = battery.customize(T, w, D).export()
    tune.set(T, "battery_pool", 1000)
    tune.set(T, "battery_buffer", 64)
    got = battery.customize(T, w, D).export()
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    with pytest.raises(Exception):
        tune.set(T, "battery_buffer", 8)


def test_battery_drop_in(gpu):
    """nwcch.cch_nb_battery has the reference's names, arguments and layout:
    the 8 arrays hold the reference's profiles, battery_query its answers."""
    from nwcch import cch_nb_battery as nbb
    g, caps = battery_cases()[3]
    c = caps[1]
    prof = nbb.battery_customize(int(g["n"]), g["first"], g["head"], g["e_arc"], g["e_up"].astype(bool), g["w"],
                                 float(c["M"]))
    cnt, I1, C1, O1, pst, PI, PC, PO = prof
    assert np.array_equal(cnt, c["cnt"])
    for d in range(cnt.size):
        want = c["pieces"][c["poff"][d]:c["poff"][d + 1]]
        if cnt[d] == 1:
            assert (I1[d], C1[d], O1[d]) == tuple(want[0])
        elif cnt[d] > 1:
            p0 = pst[d]
            got = np.stack([PI[p0:p0 + cnt[d]], PC[p0:p0 + cnt[d]], PO[p0:p0 + cnt[d]]], axis=1)
            assert np.array_equal(got, want)
    soc = dsoc = mark = None
    for j in range(5):
        s, t = g["rank"][c["qs"][j]], g["rank"][c["qt"][j]]
        b = nbb.battery_query(s, t, c["b0"][j], g["first"], g["head"], g["parent"], *prof, soc, dsoc, mark, j + 1)
        assert b == c["ans"][j]
    h = nbb.size_histogram(cnt)
    assert h[:7].sum() == cnt.size and h[7] == cnt.max()


def test_battery_cch_class(gpu):
    """nwcch.cch_battery.BatteryCCH (python/cch_battery.py's class shape)
    over nwcch.cch.CCH with the fixture's order: the reference's profiles,
    answers by original vertex ids, the reference's (largest, mean) pair."""
    from nwcch.cch import CCH
    from nwcch.cch_battery import BatteryCCH
    g, caps = battery_cases()[4]
    c = CCH(int(g["n"]), g["off"], g["tgt"], order=g["rank"])
    assert np.array_equal(c.first, g["first"]) and np.array_equal(c.head, g["head"])
    bc = BatteryCCH(c)
    for cap in caps:
        largest, mean = bc.customize(g["w"], float(cap["M"]))
        assert largest == int(cap["cnt"].max())
        assert abs(mean - cap["poff"][-1] / cap["cnt"].size) < 1e-12
        up, down = bc.profiles()
        for a in (0, len(up) // 2, len(up) - 1):
            assert up[a] == [tuple(p) for p in cap["pieces"][cap["poff"][2 * a]:cap["poff"][2 * a + 1]]]
            assert down[a] == [tuple(p) for p in cap["pieces"][cap["poff"][2 * a + 1]:cap["poff"][2 * a + 2]]]
        got = bc.query_batch(cap["qs"], cap["qt"], cap["b0"])
        assert np.array_equal(got, cap["ans"])
        assert bc.query(int(cap["qs"][0]), int(cap["qt"][0]), float(cap["b0"][0])) == cap["ans"][0]


def test_battery_edges(gpu):
    """A single vertex, an empty query batch, capacity 0 (only free arcs and
    recuperation are feasible) and out-of-range ids."""
    import oracle as orc
    from nwcch import _lib, battery
    from nwcch.device import DeviceTopology
    T1 = DeviceTopology(1, np.zeros(2, np.int64), np.zeros(0, np.int32), np.array([-1]), np.zeros(0, np.int64),
                        np.zeros(0, np.int8))
    b1 = battery.customize(T1, np.zeros(0), 5.0)
    assert b1.pieces == 0
    assert b1.query([0], [0], 2.5).cpu().numpy()[0] == 2.5
    assert b1.query([], [], 1.0).numel() == 0
    g, caps = battery_cases()[0]
    T = dev_topo(g)
    OT = orc.Topo(int(g["n"]), g["first"], g["head"], g["parent"], g["e_arc"], g["e_up"])
    b = battery.customize(T, g["w"], 0.0)
    want = orc.battery_customize(OT, g["w"], 0.0)
    for a, o in zip(b.export(), want):
        assert np.array_equal(a, o)
    with pytest.raises(_lib.NwcchError):
        b.query([int(g["n"])], [0], 0.0)
    with pytest.raises(_lib.NwcchError):
        battery.customize(T, g["w"], float("nan"))

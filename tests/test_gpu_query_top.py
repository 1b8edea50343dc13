"""The batched query pipeline (csrc/query_top.cu): the lower part of every
chain per warp, the top supernodes as (min,+) products over tiles of chains,
the meet per query. Its answers must equal the oracle's ET query
(python/cch_nb.py:577-615 restated) and the per-warp kernel's exactly, for
every size of the top set, for forests (pairs in different trees have no
path), s == t, several passes per batch, and metrics whose values need the
64-bit labels (the pipeline then leaves the batch to the 64-bit kernel)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _graph(kind, n, seed):
    from nwcch import graphs as G
    from nwcch import topology as TT
    if kind == "grid":
        g = G.grid(64, seed=seed)
    else:
        g = {"delaunay": G.delaunay, "road": G.road_like}[kind](n, seed=seed)
    return g, TT.build_topology(g)


@pytest.mark.parametrize("kind,n", [("road", 80_000), ("delaunay", 50_000), ("grid", 4096)])
def test_top_pipeline_equals_oracle_and_per_warp(gpu, oracle, kind, n, monkeypatch):
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph(kind, n, seed=41)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, g["w"])
    s, t = G.random_pairs(g["n"], 6000, seed=12)
    s, t = top["rank"][s].copy(), top["rank"][t].copy()
    s[:40] = t[:40]  # s == t
    t[40:80] = top["parent"][s[40:80]].clip(0)  # t an ancestor of s (the meet at the lowest rows)
    want = oracle.query_batch(OT, oup, odn, s, t)
    m = T.customize(g["w"], "int32")
    tune.set(T, "query_top_chains", 0)
    per_warp = T.query_batch(m, s, t).cpu().numpy()
    assert np.array_equal(per_warp, want)
    for chains in (1, 8, 64, 4096):  # top sets from most of the tree to none
        tune.set(T, "query_top_chains", chains)
        assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want), chains
    # several passes over one batch (label rows of 1,000 queries at a time)
    monkeypatch.setenv("NWCCH_QUERY_TOP_PASS_QUERIES", "1000")
    tune.set(T, "query_top_chains", 8)
    assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want)
    assert not T.check()


def test_top_pipeline_on_a_forest(gpu, oracle):
    """The union of the reference's technique graphs: many small trees, most
    pairs in different trees (no path: infinity)."""
    from nwcch.device import DeviceTopology
    from nwcch import tune
    z = load_golden("techniques.npz")
    T = DeviceTopology(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    OT = oracle.Topo(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"])
    oup, odn = oracle.customize(OT, z["w"])
    rng = np.random.default_rng(3)
    n = int(z["n"])
    s = rng.integers(0, n, 5000)
    t = np.where(rng.random(5000) < 0.5, rng.integers(0, n, 5000), np.clip(s + rng.integers(-2, 3, 5000), 0, n - 1))
    want = oracle.query_batch(OT, oup, odn, s, t)
    assert (want == oracle.INF).any() and (want != oracle.INF).any()
    m = T.customize(z["w"], "int32")
    for chains in (1, 64):
        tune.set(T, "query_top_chains", chains)
        assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want), chains


def test_top_pipeline_leaves_wide_values_to_the_64_bit_kernel(gpu, oracle):
    """Weights near 2^27 put label sums outside +-2^28: every kernel of the
    pipeline returns at once and the 64-bit kernel answers the batch."""
    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph("road", 30_000, seed=5)
    w = (g["w"].astype(np.int64) * 5000).astype(np.int32)
    T = DeviceTopology.from_dict(top)
    OT = oracle.Topo.from_dict(top)
    oup, odn = oracle.customize(OT, w)
    depth = int(T.depth)
    finite = np.concatenate([oup[oup != oracle.INF], odn[odn != oracle.INF]])
    assert np.abs(finite).max() * (depth + 2) > (1 << 28)  # outside the 32-bit label bound
    assert np.abs(finite).max() < (1 << 30)  # but stored in int32 without saturation
    s, t = G.random_pairs(g["n"], 3000, seed=2)
    s, t = top["rank"][s], top["rank"][t]
    want = oracle.query_batch(OT, oup, odn, s, t)
    m = T.customize(w, "int32")
    tune.set(T, "query_top_chains", 4)
    assert np.array_equal(T.query_batch(m, s, t).cpu().numpy(), want)


def test_top_pipeline_concurrent_streams(gpu):
    """Batches of several metrics enqueued at once from threads on their own
    streams (as the serving loop does): each call carves its scratch from its
    own stream-ordered allocation, so every answer equals the same batch run
    alone."""
    import threading

    import torch

    from nwcch import graphs as G
    from nwcch import tune
    from nwcch.device import DeviceTopology
    g, top = _graph("delaunay", 60_000, seed=9)
    T = DeviceTopology.from_dict(top)
    tune.set(T, "query_top_chains", 64)
    W = G.scaled_metrics(g, 4, seed=3)
    ms = [T.customize(w, "int32") for w in W]
    rng = np.random.default_rng(4)
    batches = [(top["rank"][rng.integers(0, g["n"], nq)], top["rank"][rng.integers(0, g["n"], nq)])
               for nq in (1300, 2100, 3500, 5000, 8000, 1800)]
    want = {(j, b): T.query_batch(ms[j], *batches[b]).cpu().numpy() for j in range(4) for b in range(len(batches))}
    errors, got = [], {}

    def worker(j):
        stream = torch.cuda.Stream()
        try:
            with torch.cuda.stream(stream):
                for rep in range(3):
                    for b in range(len(batches)):
                        got[j, b, rep] = T.query_batch(ms[j], *batches[b]).cpu().numpy()
        except Exception as exc:  # reported below
            errors.append(f"{type(exc).__name__}: {exc}")

    threads = [threading.Thread(target=worker, args=(j,)) for j in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors[:3]
    for (j, b, rep), d in got.items():
        assert np.array_equal(d, want[j, b]), (j, b, rep)

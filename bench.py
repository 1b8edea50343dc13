"""Benchmark of the metric-dependent CCH hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload usa24m|delaunay264k|grid64]

One step = one pass of the hot path over one batch of synthetic input: the
full customization of one metric plus the negative-cycle scan, then one batch
of elimination-tree queries on a resident customized metric. `value` is the
customization + scan time per metric in ms (lower is better), device-timed
with CUDA events over the K timed steps; query throughput, latency
percentiles, the plain per-level customization and the CPU baseline ride
along in the same JSON line.

--impl reference times the reference algorithm on the host cores: the C
restatement of cpp/cch.cpp in oracle/ (the reference checkout does not travel
to the GPU host), level-parallel customization on every core plus the scan,
on the same workload and metric.

Multi-GPU (torchrun, one rank per GPU): replicas only. Every rank customizes
its own copy of the metric over the same topology; a single metric's
customization is not sharded. Barrier + max over ranks; value = max time /
(K * N).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "negative-weight-cch_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "customize ms & batched ET queries/s vs plain at 24M nodes; p50/p99 latency"
UNIT = "ms per metric (customization + negative-cycle scan)"

WORKLOADS = {
    # USA scale: 24M-vertex road-like planar graph (Delaunay EMST + random
    # Delaunay edges up to 58.3M arcs), one injected negative 3-cycle
    "usa24m": dict(kind="road", n=24_000_000, arcs=58_333_344, queries=100_000, inject=True),
    # plain GPU configuration: 264k-vertex Delaunay graph
    "delaunay264k": dict(kind="delaunay", n=264_000, queries=10_000, inject=False),
    # a third of USA scale (8M vertices, same arcs per vertex): profiling case
    # with a working set above L2 and a few GB on the device
    "road8m": dict(kind="road", n=8_000_000, arcs=19_444_448, queries=10_000, inject=True),
    # serving configuration: 1.1M-vertex Delaunay graph, 8 resident metrics
    "delaunay1m": dict(kind="delaunay", n=1_100_000, queries=10_000, inject=False),
    # CPU configuration: 64x64 grid
    "grid64": dict(kind="grid", n=4096, queries=1_000, inject=False),
    # battery-constrained profiles in the default run (a quarter of the 264k
    # case, whose CPU reference takes about a minute per capacity)
    "delaunay66k": dict(kind="delaunay", n=66_000, queries=1_000, inject=False),
}


def log(msg):
    if int(os.environ.get("RANK", "0")) == 0:
        print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


# --------------------------------------------------------------- workload

def _cache_key(name: str, seed: int) -> str:
    """Names what a cached workload was built from: its spec, seed and the
    sources of the generators and the host preprocessing."""
    import hashlib
    h = hashlib.sha256(json.dumps([name, seed, WORKLOADS[name]], sort_keys=True).encode())
    pkg = ROOT / "negative-weight-cch_gb300"
    for p in [pkg / "nwcch" / "graphs.py", pkg / "nwcch" / "delaunay.py", pkg / "nwcch" / "topology.py",
              *sorted((pkg / "csrc").glob("host_*"))]:
        h.update(p.read_bytes())
    return h.hexdigest()[:32]


def make_workload(name: str, seed: int = 0):
    """Graph, topology (order, symbolic contraction, arc map: host C++ in
    libnwcch_host.so, no device code), metrics and query pairs of a workload.
    Workloads of 1M vertices and more are cached under NWCCH_CACHE_DIR
    (default _cache/ beside this file), so a second run on the same machine
    skips the minutes the 24M topology takes to build."""
    from nwcch import graphs as G
    from nwcch import topology as T
    spec = WORKLOADS[name]
    cache = None
    if spec["n"] >= 1_000_000 and os.environ.get("NWCCH_CACHE_DIR", "x") != "":
        cache = Path(os.environ.get("NWCCH_CACHE_DIR", str(ROOT / "_cache"))) / f"{name}_seed{seed}"
    key = _cache_key(name, seed) if cache else None
    hit = T.load_cache(cache, key) if cache else None
    if hit is not None:
        g, top = hit
        log(f"graph {g['kind']} + topology from {cache}: n={g['n']:,} arcs={g['tgt'].size:,} "
            f"m+={top['head'].size:,}")
    else:
        t0 = time.time()
        if spec["kind"] == "grid":
            g = G.grid(64, seed=seed)
        elif spec["kind"] == "delaunay":
            g = G.delaunay(spec["n"], seed=seed)
        else:
            g = G.road_like(spec["n"], arcs=spec["arcs"], seed=seed)
        log(f"graph {g['kind']}: n={g['n']:,} arcs={g['tgt'].size:,} ({time.time() - t0:.1f}s)")
        t0 = time.time()
        top = T.build_topology(g)
        log(f"order + symbolic + arc map: m+={top['head'].size:,} ({time.time() - t0:.1f}s)")
        if cache:
            t0 = time.time()
            ok = T.save_cache(cache, key, g, top)
            log(f"topology cache {'written' if ok else 'not written'}: {cache} ({time.time() - t0:.1f}s)")
    w_bad, cyc = None, None
    if spec["inject"]:
        gb, cyc = G.inject_negative_triangle(g, seed=seed + 1)
        w_bad = gb["w"]
    s, t = G.random_pairs(g["n"], spec["queries"], seed=7)
    return dict(name=name, spec=spec, g=g, top=top, w=g["w"], w_bad=w_bad, cycle=cyc,
                qs=top["rank"][s].astype(np.int32), qt=top["rank"][t].astype(np.int32))


def algorithmic_bytes(n, m, m_plus, triangles, s_w=4):
    """Per customization: every lower triangle reads up/dn of its two lower
    arcs plus a head (4 s_w + 4), every arc is initialised and written back
    with its head (4 s_w + 4), plus first[] and the original arcs (tgt,
    e_arc, e_up, w)."""
    return triangles * (4 * s_w + 4) + m_plus * (4 * s_w + 4) + 8 * (n + 1) + m * (4 + 8 + 1 + 4)


# DRAM bytes (read + write) of one customization, from one ncu capture of
# `bench.py --profile customize` on the workload (dram__bytes_read.sum +
# dram__bytes_write.sum over the customization's launches; the capture's
# summary is profiles/customize_usa24m_launches_dram.md).


def peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# --------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (reads only)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                parts = [p.strip() for p in out.stdout.strip().split(",")]
                if len(parts) == 7:
                    self.samples.append(parts)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(s[0]) for s in self.samples) if v is not None]
        mx = [v for v in (num(s[1]) for s in self.samples) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# --------------------------------------------------------------- ours

def max_over_ranks(values, device):
    """Element-wise maximum of per-rank values over the process group (the
    replicas' timings: the slowest rank sets the job's time)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def replica_units(steps: int, world: int) -> int:
    """Customizations the whole job performed: every rank customizes its own
    replica once per step."""
    return steps * world


def run_ours(args, W, world):
    import torch

    from nwcch.device import DeviceTopology
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    top = W["top"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    T = DeviceTopology.from_dict(top)  # upload + the derived arrays on the device + supernodal plan
    torch.cuda.synchronize()
    topo_s = time.perf_counter() - t0
    log(f"topology handle: {topo_s:.2f}s")
    stream = torch.cuda.current_stream()
    w_step = W["w_bad"] if W["w_bad"] is not None else W["w"]
    w_host = torch.from_numpy(w_step).pin_memory()
    w_dev = w_host.to(dev)
    good = T.customize(W["w"], "int32")                 # resident metric for the queries
    metric = T.customize(w_dev, "int32")
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    qs = torch.from_numpy(W["qs"]).to(dev)
    qt = torch.from_numpy(W["qt"]).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    fits_l2 = T.m_plus * 8 < 129e6

    # gate: the injected negative cycle is detected, the conservative metric is clean
    neg = T.negative_cycle_arcs(metric)
    if W["w_bad"] is not None:
        assert neg > 0, "injected negative cycle not detected"
    assert T.negative_cycle_arcs(good) == 0
    # the autotuner picks the customization and query schedules on this workload
    tuned = cust_tuned = None
    if not args.no_tune:
        from nwcch import tune
        rc = tune.tune_customize(T, w_dev, caps=(0, 256, 512), min_counts=(0, 1024), reps=2)
        cust_tuned = {**rc["best"], "default_ms": next(x["ms"] for x in rc["trials"]
                                                        if x["sn_warp_cap"] == 512 and x["sn_warp_min_count"] == 1024)}
        log(f"customization schedule: {cust_tuned}")
        k = min(W["qs"].size, 8192)
        r = tune.tune_queries(T, good, W["qs"][:k], W["qt"][:k], reps=2)
        tuned = {"sample_queries": k, **r["best"], "sample_ms": r["ms"],
                 "default_ms": next(x["ms"] for x in r["trials"] if x["query_dense_rows"] == 16
                                    and x["query_occupancy"] == 1 and x["labels"] == "auto")}
        rl = tune.tune_latency(T, good, W["qs"][-16:], W["qt"][-16:])
        tuned["single_query"] = rl["best"]
        log(f"query schedule: {tuned}")

    def step(ev0=None, ev1=None):
        if ev0 is not None:
            ev0.record(stream)
        T.customize(w_dev, "int32", out=metric, sync=False)
        T.negative_cycle_arcs_async(metric, count)
        if ev1 is not None:
            ev1.record(stream)

    for _ in range(args.warmup):
        step()
        T.query_batch(good, qs, qt)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    cust_ms, q_ms = [], []
    with ClockSampler(dev.index) as clocks:
        torch.cuda.synchronize()
        t_all = time.perf_counter()
        for _ in range(args.steps):
            if fits_l2:
                flush.fill_(1)  # working set below L2: flush between steps (untimed)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            step(e0, e1)
            T.query_batch(good, qs, qt)  # synchronizes
            q_launches = T.last_query_launches()
            e2.record(stream)
            torch.cuda.synchronize()
            cust_ms.append(e0.elapsed_time(e1))
            q_ms.append(e1.elapsed_time(e2))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t_all
    if world > 1:
        torch.distributed.barrier()
    sat = T.check()
    neg_k = int(count.item())
    # the plain per-level form of the same customization
    plain_ms = []
    same = None
    plain_steps = args.plain_steps if args.plain_steps >= 0 else (0 if T.n > 5_000_000 else 1)
    if plain_steps:
        plain = T.customize(w_dev, "int32", method="plain")
        for _ in range(plain_steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            T.customize(w_dev, "int32", out=plain, sync=False, method="plain")
            e1.record(stream)
            torch.cuda.synchronize()
            plain_ms.append(e0.elapsed_time(e1))
        same = bool(torch.equal(plain.up, metric.up) and torch.equal(plain.dn, metric.dn))
        del plain
    # the plain per-query form on the same batch (one ancestor at a time)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ref_d = T.query_batch(good, qs, qt)
    e0.record(stream)
    plain_d = T.query_batch(good, qs, qt, method="plain")
    e1.record(stream)
    torch.cuda.synchronize()
    plain_q_ms = e0.elapsed_time(e1)
    assert torch.equal(ref_d, plain_d), "batched and plain queries differ"
    # the same batch as one captured CUDA graph, replayed
    graph_q = None
    try:
        qg = T.query_graph(good, int(qs.numel()))
        gms = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            gd = qg.run(qs, qt)
            e1.record(stream)
            torch.cuda.synchronize()
            gms.append(e0.elapsed_time(e1))
        assert torch.equal(gd, ref_d), "graph-replayed and direct queries differ"
        graph_q = {"ms": round(statistics.median(gms), 4),
                   "queries_per_s": round(qs.numel() / (statistics.median(gms) / 1000), 1)}
        del qg
    except Exception as exc:  # reported, not fatal: the direct form is the measured one
        graph_q = {"error": f"{type(exc).__name__}: {exc}"[:200]}
    # end to end through the public API: weights from pinned host memory,
    # customization, scan, count read back
    e2e_ms = []
    for _ in range(max(3, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w_dev.copy_(w_host, non_blocking=True)
        T.customize(w_dev, "int32", out=metric, sync=False)
        T.negative_cycle_arcs_async(metric, count)
        c = int(count.item())
        e2e_ms.append((time.perf_counter() - t0) * 1000)
        assert c == neg_k
    # single-query latency (one query per call)
    lat, lat_dist = [], []
    for i in range(min(200, W["qs"].size)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d1 = T.query_batch(good, qs[i:i + 1], qt[i:i + 1])
        lat.append((time.perf_counter() - t0) * 1e6)
        lat_dist.append(int(d1[0]))
    lat_dist = np.array(lat_dist, np.int64)
    # the CCH potential of the conservative metric (two sweeps)
    pot_ms = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pot = T.potential(good)
        e1.record(stream)
        torch.cuda.synchronize()
        pot_ms.append(e0.elapsed_time(e1))
    good_host = good.to_numpy()
    bad_host = metric.to_numpy()  # the timed metric, compared with the oracle's in full
    return dict(T=T, tuned=tuned, cust_tuned=cust_tuned, cust_ms=cust_ms, q_ms=q_ms, wall=wall, plain_ms=plain_ms, plain_equal=same,
                e2e_ms=e2e_ms, graph_q=graph_q, bad_host=bad_host, batch_dist=ref_d.cpu().numpy(), topo_s=topo_s,
                plain_q_ms=plain_q_ms, lat_dist=lat_dist, pot_ms=pot_ms, pot=pot.cpu().numpy(), good_host=good_host,
                lat_us=lat, clocks=clocks.summary(), neg=neg_k, saturated=bool(sat), query_launches=q_launches,
                good=good)


def scanned_arcs(top, qs, qt, sample: int = 1000) -> float:
    """Mean arcs a query relaxes in the reference's ET sweep
    (python/cch_nb.py:577-615: every arc out of every ancestor of s, then of
    t), over the first `sample` pairs of the batch: the (min,+) relaxations
    per query, walked supernode by supernode (a supernode's rows from the
    entry row x hold first[last + 1] - first[x] arcs)."""
    first = np.asarray(top["first"], np.int64)
    parent = np.asarray(top["parent"], np.int64)
    n = int(top["n"])
    rl = np.diff(first)
    join = np.zeros(n, bool)
    join[1:] = (parent[:-1] == np.arange(1, n)) & (rl[:-1] == rl[1:] + 1)
    sid = np.cumsum(~join) - 1
    s0 = np.nonzero(~join)[0]
    last = np.append(s0[1:], n) - 1
    total = 0
    k = min(sample, len(qs))
    for x in np.concatenate([qs[:k], qt[:k]]).astype(np.int64):
        while x >= 0:
            S = sid[x]
            total += int(first[last[S] + 1] - first[x])
            x = int(parent[last[S]])
    return total / max(1, k)


def cpu_potential(W, good_host, pot_dev):
    """The oracle's two-sweep potential (single thread, like the reference's
    cch_potential) on the same customized metric; equal to the device's."""
    import oracle as orc
    OT = orc.Topo.from_dict(W["top"])
    t0 = time.perf_counter()
    p = orc.potential(OT, *good_host)
    ms = (time.perf_counter() - t0) * 1000
    return dict(ms=ms, equal=bool(np.array_equal(p, pot_dev)))


def cpu_queries(W, good_host, count: int = 200):
    """The oracle's ET query (python/cch_nb.py:577-615 as plain C), one
    thread, one query after another, on the same metric and pairs: the CPU
    per-query latency beside the device's."""
    import oracle as orc
    OT = orc.Topo.from_dict(W["top"])
    s, t = W["qs"][:count].astype(np.int64), W["qt"][:count].astype(np.int64)
    t0 = time.perf_counter()
    d = orc.query_batch(OT, *good_host, s, t, threads=1)
    ms = (time.perf_counter() - t0) * 1000 / max(1, s.size)
    return dict(ms_per_query=ms, queries=int(s.size), dist=d)


def run_battery(args, Wb, factors=(0.25, 1.0, 4.0), queries: int = 10_000):
    """Battery-constrained profiles (python/run_nb_battery.py:62-117 as the
    protocol): EV energies on the workload's graph, D = median unconstrained
    energy of random reachable pairs, capacities M = 0.25 D, D, 4 D; per M
    the customization (device time, warm), the profile sizes, and a batch of
    queries with b0 = M and M / 2 per pair."""
    import torch

    from nwcch import battery
    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    g, top = Wb["g"], Wb["top"]
    w = G.ev_energies(g)
    T = DeviceTopology.from_dict(top)
    wt = battery.energies(T, w)
    # D from the battery path itself: a capacity far above any route's energy
    # and half of it as the start charge make every query unconstrained
    big = 1e12
    s, t = G.random_pairs(g["n"], 400, seed=21)
    free = battery.customize(T, wt, big)
    soc = free.query(top["rank"][s], top["rank"][t], big / 2).cpu().numpy()
    free.free()
    reach = soc > -np.inf
    D = float(np.median((big / 2 - soc[reach])[:50]))
    qs, qt = G.random_pairs(g["n"], queries // 2, seed=23)
    qs = np.repeat(top["rank"][qs], 2).astype(np.int32)
    qt = np.repeat(top["rank"][qt], 2).astype(np.int32)
    sq, tq = torch.from_numpy(qs).cuda(), torch.from_numpy(qt).cuda()
    out = []
    for f in factors:
        M = f * D
        b0 = torch.from_numpy(np.tile([M, M / 2], queries // 2)).cuda()
        times = []
        reps = max(1, min(args.steps, 2))
        for rep in range(1 + reps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            b = battery.customize(T, wt, M)
            e1.record()
            torch.cuda.synchronize()
            if rep:
                times.append(e0.elapsed_time(e1))
            if rep < reps:
                b.free()
        res = b.query(sq, tq, b0)
        qms = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            b.query(sq, tq, b0, out=res, sync=False)
            e1.record()
            torch.cuda.synchronize()
            qms.append(e0.elapsed_time(e1))
        lat = []
        for j in range(50):
            t0 = time.perf_counter()
            b.query(sq[j:j + 1], tq[j:j + 1], b0[j:j + 1])
            lat.append((time.perf_counter() - t0) * 1e6)
        lat.sort()
        r = res.cpu().numpy()
        out.append({"factor": f, "M": M, "customize_ms": round(statistics.median(times), 3),
                    "pieces": b.pieces, "largest_profile": b.largest,
                    "size_histogram": [int(v) for v in b.size_histogram()],
                    "queries": int(qs.size), "queries_per_s": round(qs.size / (statistics.median(qms) / 1000), 1),
                    "query_latency_us": {"p50": round(lat[len(lat) // 2], 1), "p99": round(lat[-1], 1)},
                    "infeasible": int(np.count_nonzero(r == -np.inf)), "_profiles": b, "_answers": r,
                    "_b0": b0.cpu().numpy()})
    return {"workload": Wb["name"], "energies": "EV model: L + 1.0 x climb - 0.6 x descent (float64)",
            "D": D, "capacities": out, "_T": T, "_w": w, "_qs": qs, "_qt": qt}


def cpu_battery(Wb, B, budget_s: float = 30.0):
    """The oracle's battery customization (python/cch_nb_battery.py:48-183
    as plain C, one thread) at M = D, and its queries on the same pairs;
    checks the device profiles and answers against it."""
    import oracle as orc
    OT = orc.Topo.from_dict(Wb["top"])
    cap = next(c for c in B["capacities"] if c["factor"] == 1.0)
    t0 = time.perf_counter()
    prof = orc.battery_customize(OT, B["_w"], cap["M"])
    cust_s = time.perf_counter() - t0
    dev = cap["_profiles"].export()
    equal = all(np.array_equal(a, b) for a, b in zip(dev, prof))
    n = max(1, min(B["_qs"].size, int(budget_s / max(cust_s, 1e-3) * 200)))
    t0 = time.perf_counter()
    ans = orc.battery_query_batch(OT, prof, B["_qs"][:n], B["_qt"][:n], cap["_b0"][:n], threads=1)
    qs_s = time.perf_counter() - t0
    return {"customize_s_M_eq_D": round(cust_s, 3), "queries": n,
            "queries_per_s_1_thread": round(n / qs_s, 1), "threads": 1,
            "profiles_equal_device": bool(equal),
            "answers_equal_device": bool(np.array_equal(ans, cap["_answers"][:n]))}


def batched_bytes(n, m, m_plus, triangles, k, s_w=4):
    """Per batched customization of k metrics: the topology (heads, first,
    arc map) is read once, weights and up/dn once per metric."""
    return (triangles * (4 * s_w * k + 4) + m_plus * (4 * s_w * k + 4) + 8 * (n + 1)
            + m * (8 + 1 + 4 + 4 * k))


def run_updates(T, m, top, new_weights, sizes, reps, cpu_budget_s, seed):
    """Partial re-customizations (python/cch.py:349-402) of `size` random
    original arcs of the resident metric m, `reps` per size, sizes in
    ascending order. Each is timed on the host around the public call (the
    statistics read back included) and with CUDA events, and checked equal to
    a full customization of the new weights. The oracle's update runs the
    same changes from the same arrays on one core, on the reference's update
    index built once (python/cch.py:289-290), while its time stays within
    cpu_budget_s: each compared in evaluated count and changed set, and the
    arrays compared in full when it followed every update."""
    import torch

    import oracle as orc
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(seed)
    OT = orc.Topo.from_dict(top)
    t0 = time.perf_counter()
    X = orc.UpdateIndex(OT)
    index_s = time.perf_counter() - t0
    w_o = m.w.cpu().numpy().astype(np.int32)
    up_o, dn_o = m.to_numpy()
    full = T.customize(m.w, m.storage)
    cpu_on, cpu_spent, checked, oracle_equal = True, 0.0, 0, True
    out = {}
    for size in sizes:
        wall, dev_ms, ev, cpu = [], [], [], []
        for _ in range(reps):
            idx = rng.choice(T.m, size=size, replace=False)
            val = new_weights(idx, rng)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record(stream)
            ev.append(T.update(m, idx, val))
            e1.record(stream)
            torch.cuda.synchronize()
            wall.append((time.perf_counter() - t0) * 1000)
            dev_ms.append(e0.elapsed_time(e1))
            assert m.stats["changed_negative"] == 0
            T.customize(m.w, m.storage, out=full)
            assert torch.equal(full.up, m.up) and torch.equal(full.dn, m.dn), "partial != full recompute"
            if cpu_on:
                ch = np.sort(m.last_changed.cpu().numpy().astype(np.int64))
                t0 = time.perf_counter()
                oev, och, _ = X.update(w_o, up_o, dn_o, idx, val)
                dt = time.perf_counter() - t0
                cpu.append(dt * 1000)
                cpu_spent += dt
                checked += 1
                oracle_equal &= bool(oev == ev[-1] and np.array_equal(np.sort(och), ch))
                cpu_on = cpu_spent <= cpu_budget_s
        out[str(size)] = {"ms_median": round(statistics.median(wall), 3),
                          "device_ms_median": round(statistics.median(dev_ms), 3),
                          "evaluated_median": int(statistics.median(ev)), "reps": reps,
                          "cpu_ms_median": round(statistics.median(cpu), 3) if cpu else None,
                          "cpu_reps": len(cpu)}
    arrays_equal = None
    if cpu_on:
        up, dn = m.to_numpy()
        arrays_equal = bool(np.array_equal(up, up_o) and np.array_equal(dn, dn_o))
        oracle_equal &= arrays_equal
    X.close()
    del full
    return {"sizes": out, "equal_full_recompute": True, "oracle_checked": checked, "oracle_equal": oracle_equal,
            "oracle_arrays_equal_after_last": arrays_equal,
            "cpu": {"kind": "port", "cores": 1, "index_build_s": round(index_s, 3),
                    "sample": f"the oracle's update (python/cch.py:349-402) on the first {checked} changes, "
                              f"within {cpu_budget_s:g} s; index built once, outside the times"}}


def run_updates_headline(args, W, R):
    """Partial updates on the headline workload's resident conservative
    metric: the tuner's sweep budget and dense threshold for this topology
    first, then run_updates with new lengths L' in [1, 2L] (heights kept, so
    the metric stays conservative)."""
    T, m = R["T"], R["good"]
    L = W["g"]["L"].astype(np.int64)
    heights = W["w"].astype(np.int64) - L
    tuned = None
    if not args.no_tune:
        from nwcch import tune
        tuned = tune.tune_update(T, m, sizes=(1, 10, 100), factors=(0.5, 1.0, 2.0), picks_per_size=3,
                                 seed=13)["best"]
    sizes = tuple(int(x) for x in args.update_sizes.split(",") if x)
    res = run_updates(T, m, W["top"], lambda idx, rng: heights[idx] + rng.integers(1, 2 * L[idx] + 1),
                      sizes=sizes, reps=args.update_reps, cpu_budget_s=args.cpu_budget, seed=23)
    res.update(workload=W["name"], schedule=tuned, full_customize_ms=round(statistics.median(R["cust_ms"]), 3))
    return res


def run_batch(args, Wd, K):
    """K metrics of one topology customized in one batched launch sequence,
    against K single customizations of the same metrics; then partial
    re-customizations of 1, 100 and 1000 changed arcs, each checked equal to a
    full recompute."""
    import torch

    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    g, top = Wd["g"], Wd["top"]
    T = DeviceTopology.from_dict(top)
    stream = torch.cuda.current_stream()
    Wk = G.scaled_metrics(g, K, seed=11)
    w_dev = torch.from_numpy(Wk).cuda()
    b = T.customize_batch(w_dev)
    counts = T.negative_cycle_arcs_batch(b)
    torch.cuda.synchronize()
    assert int(counts.sum()) == 0, "conservative metrics reported negative cycles"
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    fits_l2 = K * T.m_plus * 8 < 129e6

    def timed(fn, steps):
        out = []
        for _ in range(steps):
            if fits_l2:
                flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return out

    def batch_step():
        T.customize_batch(w_dev, out=b, sync=False)
        T.negative_cycle_arcs_batch(b, out=counts)

    w1 = torch.empty(T.m, dtype=torch.int32, device="cuda")
    single = T.customize(w1.copy_(w_dev[0]), "int32")
    c1 = torch.zeros(1, dtype=torch.int64, device="cuda")

    def singles_step():
        for k in range(K):
            w1.copy_(w_dev[k])
            T.customize(w1, "int32", out=single, sync=False)
            T.negative_cycle_arcs_async(single, c1)

    for _ in range(max(3, args.warmup)):
        batch_step()
        singles_step()
    torch.cuda.synchronize()
    batch_ms = timed(batch_step, max(3, args.steps))
    singles_ms = timed(singles_step, 3)
    assert not T.check()
    # every metric of the batch equals its single customization
    equal = True
    for k in range(K):
        T.customize(w1.copy_(w_dev[k]), "int32", out=single, sync=False)
        equal &= bool(torch.equal(single.up, b.up[k]) and torch.equal(single.dn, b.dn[k]))
    assert equal, "batched customization differs from single customization"
    b0_host = b.metric(0).to_numpy()
    # partial re-customization of metric 0: new lengths L' in [1, 2L] keep the
    # metric conservative (w' = height difference + L')
    m0 = b.metric(0)
    L = g["L"].astype(np.int64)
    heights = Wk[0].astype(np.int64) - L  # w = length + height difference; lengths change, heights stay
    upd_tuning = None
    if not args.no_tune:
        # sweep budget and dense threshold of this topology (raise-and-restore
        # pairs on other arcs; the metric ends as it began)
        from nwcch import tune
        upd_tuning = tune.tune_update(T, m0, sizes=(1, 100, 1000), factors=(0.25, 0.5, 1.0), seed=9)["best"]
    updates = run_updates(T, m0, top, lambda idx, rng: heights[idx] + rng.integers(1, 2 * L[idx] + 1),
                          sizes=(1, 100, 1000), reps=5, cpu_budget_s=args.cpu_budget, seed=5)
    # parity at this size: metric 0 of the batch (before the updates) and 10k
    # queries on it against the oracle
    par = batch_parity(Wd, Wk[0], b0_host, qs=Wd["qs"], qt=Wd["qt"], T=T, m=b.metric(0))
    par["updates_equal_oracle"] = updates["oracle_equal"]
    par["equal"] = par["equal"] and updates["oracle_equal"]
    bm = statistics.median(batch_ms)
    B = batched_bytes(top["n"], top["e_arc"].size, T.m_plus, T.triangles, K)
    return {"workload": Wd["name"], "metrics": K, "batch_ms": round(bm, 3), "ms_per_metric": round(bm / K, 4),
            "singles_ms": round(statistics.median(singles_ms), 3),
            "speedup_vs_singles": round(statistics.median(singles_ms) / bm, 2),
            "equal_to_singles": equal, "achieved_gbs": round(B / (bm / 1000) / 1e9, 1),
            "algorithmic_bytes": int(B),
            "l2": "flushed between steps" if fits_l2 else "inputs larger than L2",
            "partial_updates": updates, "update_schedule": upd_tuning, "parity": par}


def run_batch_headline(args, W, K, single_ms):
    """K metrics of the headline workload's topology customized in one batched
    launch sequence (grid y = metric), against the single-metric time of the
    timed step; metric 0 of the batch equal to its single customization."""
    import torch

    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    T = DeviceTopology.from_dict(W["top"])
    stream = torch.cuda.current_stream()
    Wk = G.scaled_metrics(W["g"], K, seed=11)
    w_dev = torch.from_numpy(Wk).cuda()
    del Wk
    b = T.customize_batch(w_dev)
    counts = T.negative_cycle_arcs_batch(b)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(3, min(args.steps, 5))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        T.customize_batch(w_dev, out=b, sync=False)
        T.negative_cycle_arcs_batch(b, out=counts)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    assert not T.check()
    single = T.customize(w_dev[0].contiguous(), "int32")
    equal = bool(torch.equal(single.up, b.up[0]) and torch.equal(single.dn, b.dn[0]))
    assert equal, "batched customization differs from single customization"
    bm = statistics.median(times)
    out = {"workload": W["name"], "metrics": K, "batch_ms": round(bm, 3), "ms_per_metric": round(bm / K, 3),
           "single_metric_ms": round(single_ms, 3), "speedup_per_metric": round(single_ms / (bm / K), 2),
           "metric0_equal_single": equal, "negative_cycle_arcs": [int(c) for c in counts.cpu()],
           "l2": "inputs larger than L2"}
    del b, w_dev, single, T
    torch.cuda.empty_cache()
    return out


def batch_parity(Wd, w0, arcs0, qs, qt, T, m):
    """Metric 0 of the batch as customized by the device equal to the
    oracle's level-parallel customization, and the device's answers on the
    workload's query pairs (after the updates, on the updated metric) equal
    to the oracle's on the same metric."""
    import oracle as orc
    OT = orc.Topo.from_dict(Wd["top"])
    up, dn = orc.customize_parallel(OT, w0, threads=orc.cpu_count())
    cust_eq = bool(np.array_equal(up, arcs0[0]) and np.array_equal(dn, arcs0[1]))
    d_dev = T.query_batch(m, qs, qt).cpu().numpy()
    d_orc = orc.query_batch(OT, *m.to_numpy(), qs.astype(np.int64), qt.astype(np.int64), threads=orc.cpu_count())
    q_eq = bool(np.array_equal(d_dev, d_orc))
    return {"workload": Wd["name"], "customize_equal": cust_eq, "arcs_compared": int(up.size),
            "queries_checked": int(qs.size), "queries_equal": q_eq, "equal": cust_eq and q_eq}


def run_serving(args, Ws, loads):
    """8 resident metrics of one topology behind the serving loop: an open
    Poisson stream of queries (uniform s, t, metric) at each offered load,
    with update batches of 1-1000 arcs every 0.1 s on average; batched
    (supernodal) against plain per-query kernels."""
    from nwcch import graphs as G
    from nwcch.device import DeviceTopology
    from nwcch.serve import ServingLoop, poisson_trace, run_trace, summarize
    g, top = Ws["g"], Ws["top"]
    T = DeviceTopology.from_dict(top)
    W8 = G.scaled_metrics(g, 8, seed=21)
    keys = list(range(8))
    runs = []
    import torch
    tuned = None
    if not args.no_tune:
        # the autotuner on this topology: customization plan, the query
        # schedule of a serving-sized batch, the update sweep budget
        from nwcch import tune
        rc = tune.tune_customize(T, W8[0], caps=(0, 256, 512), min_counts=(0, 1024), reps=2)
        m0 = T.customize(W8[0], "int32")
        sq, tq = G.random_pairs(top["n"], 512, seed=3)
        rq = tune.tune_queries(T, m0, top["rank"][sq], top["rank"][tq], reps=2, dense_rows=(1, 8, 16),
                               labels=("auto", "shared"))
        ru = tune.tune_update(T, m0, sizes=(1, 10, 100, 1000), factors=(0.1, 0.25, 0.5, 1.0), picks_per_size=3)
        tuned = {"customize": rc["best"], "queries": rq["best"], "update_budget_ns": ru["best"]["budget_ns"],
                 "update_dense_min": ru["best"]["dense_min"]}
        log(f"serving schedules: {tuned}")
        del m0
    # one customization of this topology, for scale (events, warm)
    m0 = T.customize(W8[0], "int32")
    cms = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        T.customize(m0.w, "int32", out=m0, sync=False)
        e1.record()
        torch.cuda.synchronize()
        cms.append(e0.elapsed_time(e1))
    del m0
    for method in ("supernodal", "plain"):
        for rate in loads:
            if method == "plain" and rate > 1e5:
                continue  # the plain kernels saturate far below this load
            duration = min(args.serve_seconds, 200_000 / rate)
            shadow = {k: W8[k].copy() for k in keys}
            trace = poisson_trace(T, keys, rate, duration, update_every=0.1, update_sizes=(1, 10, 100, 1000),
                                  weights=shadow, L=g["L"], seed=int(rate) % 100_003)
            with ServingLoop(T, method=method) as loop:
                for k in keys:
                    loop.add_metric(k, W8[k])
                for b in [loop.submit_query(k, 0, 0) for k in keys]:  # admit + customize before the clock
                    b.wait(300)
                b0, q0 = loop.batches, loop.batched_queries
                res = run_trace(loop, trace)
                st = summarize(res)
                nb = loop.batches - b0
                st.update(method=method, offered_qps=rate, seconds=round(duration, 3), batches=nb,
                          mean_batch=round((loop.batched_queries - q0) / max(1, nb), 1))
            log(f"serving: {st}")
            runs.append(st)
    return {"workload": Ws["name"], "n": top["n"], "m_plus": T.m_plus, "triangles": T.triangles,
            "customize_ms": round(statistics.median(cms), 3), "schedules": tuned,
            "metrics": 8, "update_sizes": [1, 10, 100, 1000],
            "updates_per_s": 10, "latency": "scheduled arrival to answer on the host", "runs": runs}


def profile_part(args):
    """One part of the hot path on the workload, --warmup then --steps times,
    with a fixed schedule (plan parameters from the command line, default
    query schedule): a small, repeatable command for ncu captures."""
    import torch

    from nwcch import tune
    from nwcch.device import DeviceTopology
    W = make_workload(args.workload, seed=0)
    T = DeviceTopology.from_dict(W["top"])
    if args.sn_warp_cap is not None:
        tune.set(T, "sn_warp_cap", args.sn_warp_cap)
    if args.sn_warp_min_count is not None:
        tune.set(T, "sn_warp_min_count", args.sn_warp_min_count)
    if args.sn_chain_max_items is not None:
        tune.set(T, "sn_chain_max_items", args.sn_chain_max_items)
    w = torch.from_numpy(W["w"]).cuda()
    m = T.customize(w, "int32")
    qs, qt = torch.from_numpy(W["qs"]).cuda(), torch.from_numpy(W["qt"]).cuda()
    rng = np.random.default_rng(1)
    idx = rng.choice(T.m, size=100, replace=False)
    w0 = W["w"][idx].astype(np.int64)
    parts = {
        "customize": lambda i: T.customize(w, "int32", out=m, sync=False),
        "potential": lambda i: T.potential(m),
        "queries": lambda i: T.query_batch(m, qs, qt),
        "query1": lambda i: T.query_batch(m, qs[i:i + 1], qt[i:i + 1]),  # one query per call
        "update": lambda i: T.update(m, idx, w0 + (1 + i % 2)),
    }
    if args.profile == "battery":
        # battery profiles at M = D (the median unconstrained route energy,
        # read off a customization with an unbounded capacity)
        from nwcch import battery
        from nwcch import graphs as G
        wb = battery.energies(T, G.ev_energies(W["g"]))
        free = battery.customize(T, wb, 1e12)
        soc = free.query(W["qs"][:400], W["qt"][:400], 5e11).cpu().numpy()
        free.free()
        D = float(np.median((5e11 - soc[soc > -np.inf])[:50]))
        parts["battery"] = lambda i: battery.customize(T, wb, D).free()
    fn = parts[args.profile]
    for i in range(args.warmup):
        fn(i)
    torch.cuda.synchronize()
    times = []
    for i in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn(i)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    print(json.dumps({"profile": args.profile, "workload": args.workload, "ms": [round(x, 4) for x in times],
                      "sn_launches": T.sn_launches, "chain_level": T.chain_level, "chain_phases": T.chain_phases,
                      "sn_warp_cap": tune.get(T, "sn_warp_cap"),
                      "sn_warp_min_count": tune.get(T, "sn_warp_min_count")}), flush=True)


def cpu_baseline(W, budget_s: float, forms=("parallel",)):
    """The oracle ports of the reference customization plus the scan on the
    same metric, each repeated within budget_s (at least once): "serial" is
    CCH::customize (cpp/cch.cpp:437-463, one core), "parallel" the
    level-parallel customize_parallel (cpp/cch.cpp:468-529, OpenMP on every
    host core). The reference's results lead with the serial form, which is
    the faster of the two on road graphs (results/cpp_USA.txt:7,22), so
    `value` is the faster form's median. Returns the customized arcs of the
    last run for the parity check."""
    import oracle as orc
    OT = orc.Topo.from_dict(W["top"])
    cores = orc.cpu_count()
    w = W["w_bad"] if W["w_bad"] is not None else W["w"]
    res = {}
    up = dn = neg = None
    for form in forms:
        times = []
        t_start = time.perf_counter()
        while not times or (time.perf_counter() - t_start < budget_s and len(times) < 5):
            t0 = time.perf_counter()
            if form == "serial":
                up, dn = orc.customize(OT, w)
            else:
                up, dn = orc.customize_parallel(OT, w, threads=cores)
            neg = orc.negative_cycle_arcs(up, dn)
            times.append((time.perf_counter() - t0) * 1000)
        res[form] = {"ms": round(statistics.median(times), 3), "runs": len(times),
                     "cores": 1 if form == "serial" else cores}
        log(f"cpu {form} customization + scan: {res[form]}")
    best = min(res, key=lambda f: res[f]["ms"])
    return dict(value=res[best]["ms"], cores=res[best]["cores"], runs=res[best]["runs"], form=best, forms=res,
                neg=neg, up=up, dn=dn)


def check_parity(W, top_cb, device_arcs, good_host, device_dist, qs, qt, count: int):
    """Full-size parity of the benchmark's own workload (the reference
    drivers' own check, python/run_nb.py:136-141 and cpp/cch.cpp:896-903,
    against the oracle): every customized arc of the timed metric equal to
    the oracle's, and the first `count` answers of the device's query batch
    equal to the oracle's ET query on every host core."""
    import oracle as orc
    OT = orc.Topo.from_dict(W["top"])
    up, dn = device_arcs
    cust_eq = bool(np.array_equal(up, top_cb["up"]) and np.array_equal(dn, top_cb["dn"]))
    mism = 0 if cust_eq else int(np.count_nonzero(up != top_cb["up"]) + np.count_nonzero(dn != top_cb["dn"]))
    k = min(count, int(device_dist.size))
    t0 = time.perf_counter()
    d = orc.query_batch(OT, *good_host, qs[:k].astype(np.int64), qt[:k].astype(np.int64), threads=orc.cpu_count())
    q_eq = bool(np.array_equal(d, device_dist[:k]))
    out = {"workload": W["name"], "customize_equal": cust_eq, "arcs_compared": int(up.size),
           "queries_checked": int(k), "queries_equal": q_eq,
           "oracle_query_s": round(time.perf_counter() - t0, 2)}
    if not cust_eq:
        out["arcs_differing"] = mism
    if not q_eq:
        out["queries_differing"] = int(np.count_nonzero(d != device_dist[:k]))
    log(f"parity: {out}")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("NWCCH_BENCH_WORKLOAD", "usa24m"), choices=list(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--parity-queries", type=int, default=10_000,
                    help="answers of the timed query batch checked against the oracle (all host cores)")
    ap.add_argument("--batch-metrics", type=int, default=64,
                    help="metrics of the batched customization (0: skip it)")
    ap.add_argument("--batch-workload", default="delaunay264k", choices=list(WORKLOADS))
    ap.add_argument("--headline-batch-metrics", type=int, default=8,
                    help="metrics of a batched customization on the headline workload (0: skip it)")
    ap.add_argument("--update-reps", type=int, default=3,
                    help="partial updates per size on the headline workload (0: skip them)")
    ap.add_argument("--update-sizes", default="1,10,100", help="changed arcs per partial update")
    ap.add_argument("--serve-workload", default="delaunay1m", choices=list(WORKLOADS) + ["none"])
    ap.add_argument("--serve-loads", default="1e4,1e5,1e6", help="offered query loads (queries/s)")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--battery-workload", default="delaunay66k", choices=list(WORKLOADS) + ["none"],
                    help="graph of the battery-constrained profiles section")
    ap.add_argument("--no-tune", action="store_true", help="keep the default query schedule")
    ap.add_argument("--plain-steps", type=int, default=-1,
                    help="plain per-level customizations to time (-1: one, none above 5M vertices)")
    ap.add_argument("--profile", choices=["customize", "potential", "queries", "query1", "update", "battery"],
                    help="run only this part, --steps times after --warmup (for ncu captures); no bench line")
    ap.add_argument("--sn-warp-cap", type=int, default=None, help="customization plan: warp-kernel trapezoid cap")
    ap.add_argument("--sn-warp-min-count", type=int, default=None, help="customization plan: level threshold")
    ap.add_argument("--sn-chain-max-items", type=int, default=None,
                    help="customization plan: persistent launch of the levels whose launches hold at most this many "
                         "items (0: none)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.profile:
        profile_part(args)
        return
    if args.impl == "reference":
        if rank != 0:
            return
        W = make_workload(args.workload)
        cb = cpu_baseline(W, args.cpu_budget, forms=("serial", "parallel"))
        top = W["top"]
        form = {"serial": "serial CCH::customize (cpp/cch.cpp:437-463), 1 core",
                "parallel": f"level-parallel customize_parallel (cpp/cch.cpp:468-529), {cb['cores']} cores"}
        line = {"metric": METRIC, "impl": "reference", "value": round(cb["value"], 3), "unit": UNIT,
                "higher_is_better": False, "n_gpus": args.gpus, "steps": cb["runs"], "warmup": 0,
                "dtype": "int64", "data": "synthetic",
                "config": {"workload": args.workload, "n": top["n"], "arcs": int(W["g"]["tgt"].size),
                           "m_plus": int(top["head"].size),
                           "triangles": int(count_triangles(top)),
                           "negative_cycle_injected": W["w_bad"] is not None},
                "negative_cycle_arcs": cb["neg"],
                "reference_forms": cb["forms"],
                "cpu_baseline": {"value": round(cb["value"], 3), "unit": "ms", "cores": cb["cores"], "kind": "port",
                                 "sample": f"{cb['runs']} x {form[cb['form']]} + scan of the full metric "
                                           f"(the faster of the two forms; both in reference_forms)"},
                "e2e": {"value": round(cb["value"], 3), "unit": "ms", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    W = make_workload(args.workload, seed=0)
    R = run_ours(args, W, world)
    wall = R["wall"]
    cust_total = sum(R["cust_ms"]) / 1000.0
    if world > 1:
        cust_total, wall = max_over_ranks([cust_total, wall], "cuda")
    if rank != 0:
        return
    # rank 0 only, after the timed replicas: the batched and serving sections
    batch = serving = head_batch = None
    if args.headline_batch_metrics > 0:
        head_batch = run_batch_headline(args, W, args.headline_batch_metrics, statistics.median(R["cust_ms"]))
        log(f"batched (headline workload): {head_batch}")
    if args.batch_metrics > 0:
        Wd = W if args.batch_workload == args.workload else make_workload(args.batch_workload, seed=0)
        batch = run_batch(args, Wd, args.batch_metrics)
        log(f"batched: {batch}")
        del Wd
    if args.serve_workload != "none":
        Ws = W if args.serve_workload == args.workload else make_workload(args.serve_workload, seed=0)
        serving = run_serving(args, Ws, [float(x) for x in args.serve_loads.split(",") if x])
        del Ws
    bat = None
    if args.battery_workload != "none":
        Wb = W if args.battery_workload == args.workload else make_workload(args.battery_workload, seed=0)
        B = run_battery(args, Wb)
        cpu = cpu_battery(Wb, B, args.cpu_budget)
        bat = {k: v for k, v in B.items() if not k.startswith("_")}
        bat["capacities"] = [{k: v for k, v in c.items() if not k.startswith("_")} for c in B["capacities"]]
        bat["cpu_oracle"] = cpu
        log(f"battery: {bat}")
        del Wb, B
    T = R["T"]
    nq = int(W["qs"].size)
    qms = statistics.median(R["q_ms"])
    cust = statistics.median(R["cust_ms"])
    lat = sorted(R["lat_us"])
    peak, peak_src = peak_hbm()
    top = W["top"]
    B = algorithmic_bytes(top["n"], top["e_arc"].size, T.m_plus, T.triangles)
    achieved = B / (cust / 1000) / 1e9
    arcs_q = scanned_arcs(top, W["qs"], W["qt"])
    cb = cpu_baseline(W, args.cpu_budget)
    parity = check_parity(W, cb, R["bad_host"], R["good_host"], R["batch_dist"], W["qs"], W["qt"],
                          args.parity_queries)
    del cb["up"], cb["dn"]
    cp = cpu_potential(W, R["good_host"], R["pot"])
    cq = cpu_queries(W, R["good_host"])
    parity["single_queries_equal"] = bool(np.array_equal(cq["dist"], R["lat_dist"][:cq["queries"]]))
    parity["potential_equal"] = bool(cp["equal"])
    upd_head = None
    if args.update_reps > 0:
        upd_head = run_updates_headline(args, W, R)
        parity["updates_equal_oracle"] = upd_head["oracle_equal"]
        log(f"partial updates (headline workload): {upd_head}")
    if batch is not None:
        parity["batched_section"] = batch.pop("parity")
    line = {
        "metric": METRIC, "value": round(cust_total * 1000 / replica_units(args.steps, world), 4), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(cust + qms, 4), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic",
        "config": {"workload": args.workload, "n": top["n"], "arcs": int(W["g"]["tgt"].size), "m_plus": T.m_plus,
                   "triangles": T.triangles, "levels": T.levels, "depth": T.depth, "supernodes": T.supernodes,
                   "supernode_levels": T.sn_levels, "queries_per_batch": nq,
                   "negative_cycle_injected": W["w_bad"] is not None,
                   "l2": "flushed between steps" if T.m_plus * 8 < 129e6 else "inputs larger than L2",
                   "parallelism": f"replicas x{world}"},
        "customize_ms_median": round(cust, 4),
        "negative_cycle_arcs": R["neg"], "saturated": R["saturated"],
        "plain_customize_ms": round(statistics.median(R["plain_ms"]), 3) if R["plain_ms"] else None,
        "plain_equals_supernodal": R["plain_equal"],
        "queries_per_s": round(nq / (qms / 1000) * world, 1), "query_batch_ms": round(qms, 4),
        "query_work": {"arcs_per_query": round(arcs_q, 1), "sample": min(1000, nq),
                       "relaxations_per_s": round(arcs_q * nq / (qms / 1000), 1),
                       "note": "arcs of both ancestor chains (the reference's per-query relaxations); the batched "
                               "form applies each top-supernode weight to a tile of up to 32 chains"},
        # the batched query as a roofline: algorithmic bytes = one 32-bit
        # weight read per relaxation of the reference's sweep
        "query_roofline": {"bound": "hbm", "unit": "GB/s",
                           "achieved": round(4 * arcs_q * nq / (qms / 1000) / 1e9, 1),
                           "peak": peak, "frac": round(4 * arcs_q * nq / (qms / 1000) / 1e9 / peak, 4),
                           "bytes_per_query": round(4 * arcs_q, 1),
                           "note": "above 1: the tiles of the top supernodes serve each weight read to up to 32 "
                                   "chains from shared memory (L2 reads, not the reference's per-query reads)"},
        "topology_handle_s": round(R["topo_s"], 3),
        "query_schedule": R["tuned"],
        "customize_schedule": R["cust_tuned"],
        "plain_queries_per_s": round(nq / (R["plain_q_ms"] / 1000) * world, 1),
        "query_batch_graph": R["graph_q"],
        "query_latency_us": {"p50": round(lat[len(lat) // 2], 2), "p99": round(lat[max(0, int(len(lat) * 0.99) - 1)], 2),
                             "mode": "one query per call, host-timed",
                             "cpu_oracle_us_per_query": round(cq["ms_per_query"] * 1000, 2),
                             "cpu_note": "the oracle's ET query, 1 thread, same graph, metric and pairs"},
        "e2e": {"value": round(statistics.median(R["e2e_ms"]), 4), "unit": "ms",
                "h2d_bytes_per_step": int(W["w"].size * 4), "d2h_bytes_per_step": 8},
        # per timed step: k_base_gather + the supernodal launches (those
        # below the persistent top, plus k_sn_chain), the scan, and the query
        # batch's kernels
        "gpu_launches": (1 + (T.chain_from + 1 if T.chain_phases else T.sn_launches) + 1 + R["query_launches"])
                        * args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_src,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     # the DRAM bytes of a whole customization would need a
                     # counter capture of its ~1,100 launches at full size;
                     # per-kernel DRAM bytes come from single-launch captures
                     # on the 8M road-like graph instead
                     "traffic": None,
                     "traffic_note": "not captured for the whole launch graph (multi-launch counter capture at "
                                     "full size); single-launch DRAM captures of k_sn_thread and k_sn_panel on "
                                     "the 8M road-like graph are summarised with the profiles",
                     "algorithmic_bytes_per_launch": int(B),
                     "launch": "one customization: CUDA graph of k_base_gather, k_sn_thread, k_sn_warp, k_sn_panel, "
                               "k_sn_tile"},
        "cpu_baseline": {"value": round(cb["value"], 3), "unit": "ms", "cores": cb["cores"], "kind": "port",
                         "sample": f"{cb['runs']} x level-parallel customization (cpp/cch.cpp:468-529) + scan "
                                   f"of the same metric"},
        "parity": parity,
        "clocks": R["clocks"],
        "potential": {"gpu_ms": round(statistics.median(R["pot_ms"]), 3),
                      "cpu_ms": round(cp["ms"], 1), "cpu_cores": 1, "cpu_kind": "port of cpp/cch.cpp:631-655",
                      "equal": cp["equal"], "metric": "conservative (no injected cycle)"},
        "partial_updates": upd_head,
        "batched_customization": batch,
        "batched_customization_headline": head_batch,
        "serving": serving,
        "battery": bat,
    }
    print(json.dumps(line), flush=True)
    ok = (parity["customize_equal"] and parity["queries_equal"] and parity["single_queries_equal"]
          and parity["potential_equal"] and parity.get("batched_section", {}).get("equal", True)
          and parity.get("updates_equal_oracle", True))
    if not ok:
        log("PARITY FAILURE: device results differ from the oracle's")
        sys.exit(3)


def count_triangles(top) -> int:
    d = np.diff(np.asarray(top["first"], dtype=np.int64))
    return int((d * (d - 1) // 2).sum())


if __name__ == "__main__":
    main()

"""Benchmark of the metric-dependent CCH hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload usa24m|delaunay264k|grid64] [--queries Q]

One step = one pass of the hot path over one batch of synthetic input:
a full customization of one metric plus the negative-cycle scan, and one
batch of Q elimination-tree queries on a resident customized metric.
`value` is the customization + scan time per metric (ms, lower is better);
query throughput and latency percentiles ride along in the same line.

--impl reference times the reference algorithm on the host cores: the C
restatement in oracle/ (the reference checkout is not present where this
runs), level-parallel customization on every core, the scan, and the
queries, on a bounded sample of the same workload.

Multi-GPU (torchrun, one rank per GPU): every rank customizes its own
metric replica over the same topology (replicas only: one metric's
customization does not shard), barrier + max over ranks.
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

WORKLOADS = {
    # configs of the benchmark: the USA-scale road-like graph is the headline
    "usa24m": dict(kind="road", n=24_000_000, arcs=58_333_344, queries=100_000, inject=True),
    "delaunay264k": dict(kind="delaunay", n=264_000, queries=10_000, inject=False),
    "grid64": dict(kind="grid", n=4096, queries=1_000, inject=False),
}


def log(msg):
    if int(os.environ.get("RANK", "0")) == 0:
        print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


# --------------------------------------------------------------- workload

def make_workload(name: str, seed: int = 0):
    from nwcch import graphs as G
    from nwcch import topology as T
    spec = WORKLOADS[name]
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
    w_bad, cyc = (G.inject_negative_triangle(g, seed=seed + 1) if spec["inject"] else (None, None))
    s, t = G.random_pairs(g["n"], spec["queries"], seed=7)
    return dict(spec=spec, g=g, top=top, w=g["w"], w_bad=None if w_bad is None else w_bad["w"], cycle=cyc,
                qs=top["rank"][s].astype(np.int32), qt=top["rank"][t].astype(np.int32))


def algorithmic_bytes(n, m, m_plus, triangles, s_w=4):
    """Per customization: every lower triangle reads up/dn of two arcs plus a
    head, every arc is initialised and written back, plus first[] and the
    original arcs (tgt, e_arc, e_up, w)."""
    return triangles * (4 * s_w + 4) + m_plus * (4 * s_w + 4) + 8 * (n + 1) + m * (4 + 8 + 1 + 4)


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
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# --------------------------------------------------------------- ours

def run_ours(args, W, rank, world):
    import torch

    from nwcch.device import DeviceTopology
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    spec = W["spec"]
    top = W["top"]
    T = DeviceTopology.from_dict(top)
    stream = torch.cuda.current_stream()
    w_host = torch.from_numpy(W["w_bad"] if W["w_bad"] is not None else W["w"]).pin_memory()
    w_dev = w_host.to(dev)
    good = T.customize(W["w"], "int32")
    metric = T.customize(w_dev, "int32", sync=True)
    qs = torch.from_numpy(W["qs"]).to(dev)
    qt = torch.from_numpy(W["qt"]).to(dev)
    l2_flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    fits_l2 = T.m_plus * 8 < 129e6

    def step(sync_check=False):
        T.customize(w_dev, "int32", out=metric, sync=False)
        neg = T.negative_cycle_arcs(metric)
        return neg

    # correctness gate before timing: detection / exactness
    neg = T.negative_cycle_arcs(metric)
    if W["w_bad"] is not None:
        assert neg > 0, "injected negative cycle not detected"
    for _ in range(args.warmup):
        step()
        T.query_batch(good, qs, qt)
    torch.cuda.synchronize()
    # ---- timed: customization + scan (device-resident inputs)
    cust_ms = []
    with ClockSampler(dev.index) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t_all = time.perf_counter()
        for _ in range(args.steps):
            if fits_l2:
                l2_flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            T.customize(w_dev, "int32", out=metric, sync=False)
            e1.record(stream)
            neg_k = T.negative_cycle_arcs(metric)  # synchronizes
            cust_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        wall_cust = time.perf_counter() - t_all
        # ---- timed: batched queries on the resident conservative metric
        q_ms = []
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            T.query_batch(good, qs, qt)
            e1.record(stream)
            torch.cuda.synchronize()
            q_ms.append(e0.elapsed_time(e1))
    sat = T.check()
    # ---- the plain per-metric form (one launch per elimination level), for comparison
    plain_ms = []
    plain_metric = T.customize(w_dev, "int32", method="plain")
    for _ in range(args.plain_steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        T.customize(w_dev, "int32", out=plain_metric, sync=False, method="plain")
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    same = all(bool(torch.equal(a, b)) for a, b in ((plain_metric.up, metric.up), (plain_metric.dn, metric.dn)))
    # ---- e2e through the public API from pinned host memory
    e2e_ms = []
    count_host = torch.empty(1, dtype=torch.int64).pin_memory()
    for _ in range(max(2, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w_dev.copy_(w_host, non_blocking=True)
        T.customize(w_dev, "int32", out=metric, sync=False)
        c = T.negative_cycle_arcs(metric)  # device->host read of the result
        count_host[0] = c
        e2e_ms.append((time.perf_counter() - t0) * 1000)
    # ---- per-query latency sample (one query per launch)
    lat = []
    for i in range(min(200, W["qs"].size)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        T.query_batch(good, qs[i:i + 1], qt[i:i + 1])
        lat.append((time.perf_counter() - t0) * 1e6)
    res = dict(plain_ms=plain_ms, plain_equal=same, cust_ms=cust_ms, q_ms=q_ms, e2e_ms=e2e_ms, lat_us=lat, clocks=clocks.summary(), neg=neg_k,
               saturated=bool(sat or metric.saturated), wall_cust=wall_cust, T=T)
    return res


def cpu_baseline(W, budget_s=20.0):
    """The oracle port (reference algorithm in C) on the host cores."""
    import oracle as orc
    top = W["top"]
    OT = orc.Topo.from_dict(top)
    cores = orc.cpu_count()
    w = W["w_bad"] if W["w_bad"] is not None else W["w"]
    times = []
    t_start = time.perf_counter()
    while time.perf_counter() - t_start < budget_s or not times:
        t0 = time.perf_counter()
        up, dn = orc.customize_parallel(OT, w, threads=cores)
        orc.negative_cycle_arcs(up, dn)
        times.append((time.perf_counter() - t0) * 1000)
        if len(times) >= 5:
            break
    return dict(value=statistics.median(times), cores=cores, runs=len(times), up=up, dn=dn)


def roofline(W, T, cust_ms):
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peak, src = 6800.0, "fallback"
    if peaks_path.exists():
        try:
            peak = float(json.loads(peaks_path.read_text())["hbm_gbs"])
            src = "measured"
        except Exception:
            pass
    top = W["top"]
    B = algorithmic_bytes(top["n"], top["e_arc"].size, T.m_plus, T.triangles)
    dur = statistics.median(cust_ms) / 1000
    ach = B / dur / 1e9
    return {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "peak_source": src, "unit": "GB/s",
            "frac": round(ach / peak, 4), "traffic": None, "algorithmic_bytes": int(B),
            "kernel": "customization (k_base + k_pull_rows per level)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("NWCCH_BENCH_WORKLOAD", "usa24m"), choices=list(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--plain-steps", type=int, default=2)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        W = make_workload(args.workload)
        cb = cpu_baseline(W, args.cpu_budget)
        line = {"metric": METRIC, "impl": "reference", "value": round(cb["value"], 3),
                "unit": "ms (customize + negative-cycle scan, per metric)", "higher_is_better": False,
                "n_gpus": args.gpus, "steps": cb["runs"], "warmup": 0,
                "config": {"workload": args.workload, "n": W["top"]["n"], "m_plus": int(W["top"]["head"].size)},
                "cpu_baseline": {"value": round(cb["value"], 3), "unit": "ms", "cores": cb["cores"], "kind": "port",
                                 "sample": f"{cb['runs']} full level-parallel customizations + scans"},
                "e2e": {"value": round(cb["value"], 3), "unit": "ms", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    W = make_workload(args.workload, seed=0)
    R = run_ours(args, W, rank, world)
    cust = statistics.median(R["cust_ms"])
    qms = statistics.median(R["q_ms"])
    if world > 1:
        t = torch.tensor([R["wall_cust"]], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        R["wall_cust"] = float(t.item())
    if rank != 0:
        return
    T = R["T"]
    nq = W["qs"].size
    cb = cpu_baseline(W, args.cpu_budget)
    lat = sorted(R["lat_us"])
    line = {
        "metric": METRIC, "value": round(R["wall_cust"] * 1000 / (args.steps * world), 4),
        "unit": "ms (customize + negative-cycle scan, per metric)", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(cust + qms, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32 (int64 accumulation)", "data": "synthetic",
        "config": {"workload": args.workload, "n": W["top"]["n"], "arcs": int(W["g"]["tgt"].size),
                   "m_plus": T.m_plus, "triangles": T.triangles, "levels": T.levels, "depth": T.depth,
                   "queries_per_batch": nq, "negative_cycle_injected": W["w_bad"] is not None,
                   "l2": "flushed between steps" if T.m_plus * 8 < 129e6 else "inputs larger than L2",
                   "parallelism": f"replicas x{world}"},
        "customize_ms_median": round(cust, 4),
        "plain_customize_ms": round(statistics.median(R["plain_ms"]), 3) if R["plain_ms"] else None,
        "plain_equals_supernodal": R["plain_equal"],
        "supernodes": T.supernodes, "supernode_levels": T.sn_levels, "launches_per_customization": 2 + T.sn_launches,
        "negative_cycle_arcs": R["neg"], "saturated": R["saturated"],
        "queries_per_s": round(nq / (qms / 1000) * world, 1), "query_batch_ms": round(qms, 4),
        "query_latency_us": {"p50": round(lat[len(lat) // 2], 2), "p99": round(lat[int(len(lat) * 0.99) - 1], 2),
                             "mode": "one query per call, host-timed"},
        "e2e": {"value": round(statistics.median(R["e2e_ms"]), 4), "unit": "ms",
                "h2d_bytes_per_step": int(W["w"].size * 4), "d2h_bytes_per_step": 8},
        "gpu_launches": None,
        "roofline": roofline(W, T, R["cust_ms"]),
        "cpu_baseline": {"value": round(cb["value"], 3), "unit": "ms", "cores": cb["cores"], "kind": "port",
                         "sample": f"{cb['runs']} level-parallel customizations + scans of the same metric"},
        "clocks": R["clocks"],
    }
    # per customization: 2 base-value launches + the supernodal plan; 1 scan;
    # 1 launch per query batch
    line["gpu_launches"] = (2 + T.sn_launches + 1) * args.steps + args.steps
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

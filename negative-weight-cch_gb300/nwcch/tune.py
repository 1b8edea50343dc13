"""Autotuner for the schedules of one topology.

The kernels' results never depend on these choices, only their time does,
and the best choice depends on the graph (depth, supernode sizes) and the
batch size. Each tuner times its candidates on the device with CUDA events on
a sample of the caller's own workload, checks that every candidate returns
the same answers, and leaves the fastest one set on the topology
(`nwcch_tune_set`):

* customization: which small supernodes one warp customizes whole (the
  rest go through the panel and tile kernels); the plan is rebuilt for
  each candidate;
* queries: chunks below `dense_rows` rows go row by row instead of the
  32-row (min,+) form; labels in shared memory or in global scratch; the
  32-bit kernel with or without a 64-register cap; a warp or a CTA per query;
* updates: the time the level sweep may spend before the dense finish, and
  the update size from which the sweep is skipped.
"""
from __future__ import annotations

import ctypes as C
import itertools
import statistics

import numpy as np

from . import _lib
from .device import DeviceTopology, Metric

KEYS = {"query_dense_rows": 1, "query_smem_labels_max": 2, "update_budget_ns": 3, "query_occupancy": 4,
        "query_cta_max": 5, "sn_warp_cap": 6, "sn_warp_min_count": 7, "pdl": 8, "query_cta_wide_max": 9,
        "query_cta_dense_rows": 10, "battery_pool": 11, "battery_buffer": 12, "update_dense_min": 13,
        "update_spin_limit": 14, "test_barrier_extra": 15, "query_top_chains": 16, "sn_chain_max_items": 17,
        "sn_thread_cap": 18, "query_stream_max": 19, "update_small_arcs": 20,
        "update_small_ns": 21, "query_stream_ring_kb": 22}
PLAN_KEYS = {"sn_warp_cap", "sn_warp_min_count", "sn_chain_max_items", "sn_thread_cap"}

_lib.register("nwcch_tune_set", [C.c_void_p, C.c_int, C.c_int64])
_lib.register("nwcch_tune_get", [C.c_void_p, C.c_int, C.POINTER(C.c_int64)])


def get(topo: DeviceTopology, key: str) -> int:
    v = C.c_int64()
    _lib.check(_lib.lib().nwcch_tune_get(topo.handle, KEYS[key], C.byref(v)), "tune_get")
    return int(v.value)


def set(topo: DeviceTopology, key: str, value: int) -> None:  # noqa: A001 - mirrors nwcch_tune_set
    _lib.check(_lib.lib().nwcch_tune_set(topo.handle, KEYS[key], int(value)), "tune_set")
    if key in PLAN_KEYS:
        topo.refresh_info()


def tune_customize(topo: DeviceTopology, w, caps=(0, 128, 256, 512), min_counts=(0, 1024, 16384),
                   reps: int = 3, chains=(0, 1536), threads=(0, 16)) -> dict:
    """Re-plans the customization with each small-supernode schedule (which
    supernodes one warp customizes: trapezoid of at most `cap` arcs, in
    levels with at least `min_count` of them; cap 0 = none), times the
    customization of w on each (CUDA events, captured graph replayed), checks
    that the customized values never change, and keeps the fastest plan."""
    import torch
    wt = topo.weights(w)
    m = topo.customize(wt, "int32")
    ref = (m.up.clone(), m.dn.clone())
    before = (get(topo, "sn_warp_cap"), get(topo, "sn_warp_min_count"))
    cands = [(0, 0)] + [(c, k) for c in caps if c > 0 for k in min_counts]
    trials = []
    try:
        for cap, cnt in cands:
            set(topo, "sn_warp_cap", cap)
            set(topo, "sn_warp_min_count", cnt)
            ms = _time(torch, lambda: topo.customize(wt, "int32", out=m, sync=False), reps)
            if not (torch.equal(ref[0], m.up) and torch.equal(ref[1], m.dn)):
                raise AssertionError(f"customization schedule {(cap, cnt)} changed the values")
            trials.append({"sn_warp_cap": cap, "sn_warp_min_count": cnt, "ms": round(ms, 4),
                           "launches": topo.sn_launches})
    except BaseException:
        set(topo, "sn_warp_cap", before[0])
        set(topo, "sn_warp_min_count", before[1])
        raise
    best = min(trials, key=lambda r: r["ms"])
    set(topo, "sn_warp_cap", best["sn_warp_cap"])
    set(topo, "sn_warp_min_count", best["sn_warp_min_count"])
    # then the tiny supernodes of the warp levels: a thread each, or a warp
    thread_before = get(topo, "sn_thread_cap")
    thread_ms = {}
    for c in threads:
        set(topo, "sn_thread_cap", c)
        thread_ms[c] = _time(torch, lambda: topo.customize(wt, "int32", out=m, sync=False), reps)
        if not (torch.equal(ref[0], m.up) and torch.equal(ref[1], m.dn)):
            set(topo, "sn_thread_cap", thread_before)
            raise AssertionError(f"thread kernel cap {c} changed the values")
        trials.append({"sn_warp_cap": best["sn_warp_cap"], "sn_warp_min_count": best["sn_warp_min_count"],
                       "sn_thread_cap": c, "ms": round(thread_ms[c], 4), "launches": topo.sn_launches})
    if thread_ms:
        tc = min(thread_ms, key=thread_ms.get)
        set(topo, "sn_thread_cap", tc)
        best = {**best, "sn_thread_cap": tc, "ms": round(thread_ms[tc], 4)}
    # then the persistent launch of the levels near the root (0: none)
    chain_before = get(topo, "sn_chain_max_items")
    chain_ms = {}
    for c in chains:
        set(topo, "sn_chain_max_items", c)
        chain_ms[c] = _time(torch, lambda: topo.customize(wt, "int32", out=m, sync=False), reps)
        if not (torch.equal(ref[0], m.up) and torch.equal(ref[1], m.dn)):
            set(topo, "sn_chain_max_items", chain_before)
            raise AssertionError(f"persistent top launch {c} changed the values")
        trials.append({"sn_warp_cap": best["sn_warp_cap"], "sn_warp_min_count": best["sn_warp_min_count"],
                       "sn_chain_max_items": c, "ms": round(chain_ms[c], 4), "launches": topo.sn_launches,
                       "chain_level": topo.chain_level, "chain_phases": topo.chain_phases})
    if chain_ms:
        chain = min(chain_ms, key=chain_ms.get)
        set(topo, "sn_chain_max_items", chain)
        best = {**best, "sn_chain_max_items": chain, "ms": round(chain_ms[chain], 4),
                "chain_level": topo.chain_level, "chain_phases": topo.chain_phases}
    # then the launch form on the chosen plan: programmatic dependent launches
    pdl_before = get(topo, "pdl")
    forms = {}
    for pdl in (0, 1):
        set(topo, "pdl", pdl)
        forms[pdl] = _time(torch, lambda: topo.customize(wt, "int32", out=m, sync=False), reps)
        if not (torch.equal(ref[0], m.up) and torch.equal(ref[1], m.dn)):
            set(topo, "pdl", pdl_before)
            raise AssertionError(f"launch form pdl={pdl} changed the values")
        trials.append({"sn_warp_cap": best["sn_warp_cap"], "sn_warp_min_count": best["sn_warp_min_count"],
                       "sn_chain_max_items": get(topo, "sn_chain_max_items"), "pdl": pdl, "ms": round(forms[pdl], 4),
                       "launches": topo.sn_launches})
    pdl = min(forms, key=forms.get)
    set(topo, "pdl", pdl)
    best = {**best, "pdl": pdl, "ms": round(forms[pdl], 4)}
    return {"best": best, "trials": trials}


def _time(torch, fn, reps: int) -> float:
    stream = torch.cuda.current_stream()
    fn()  # warm-up (allocations, first-launch costs)
    out = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return statistics.median(out)


def tune_queries(topo: DeviceTopology, metric: Metric, s_rank, t_rank, reps: int = 3,
                 dense_rows=(1, 8, 16, 24, 33), occupancy=(1, 2, 3), labels=("auto", "global", "shared"),
                 top_chains=(16, 32, 64, 128, 256)) -> dict:
    """Times every candidate schedule on the batch (s_rank, t_rank) and keeps
    the fastest: the per-chain kernel's schedule, then the form (a warp or a
    CTA per query, or the tile pipeline of the top supernodes for large
    batches), then, when the tile pipeline answers the batch, the size of its
    top set (the supernodes crossed by about `top_chains` chains of a pass).
    Returns {"best": {...}, "ms": best time, "trials": [...]}."""
    import torch
    s = torch.as_tensor(np.asarray(s_rank, np.int32)).cuda()
    t = torch.as_tensor(np.asarray(t_rank, np.int32)).cuda()
    out = torch.empty(s.numel(), dtype=torch.int64, device="cuda")
    smem_max = {"auto": 8192, "global": 0, "shared": 1 << 40}
    before = {k: get(topo, k) for k in ("query_dense_rows", "query_smem_labels_max", "query_occupancy")}
    ref = None
    trials = []
    try:
        for dr, occ, lab in itertools.product(dense_rows, occupancy, labels):
            set(topo, "query_dense_rows", dr)
            set(topo, "query_occupancy", occ)
            set(topo, "query_smem_labels_max", smem_max[lab])
            ms = _time(torch, lambda: topo.query_batch(metric, s, t, out=out), reps)
            res = out.clone()
            if ref is None:
                ref = res
            elif not torch.equal(ref, res):
                raise AssertionError(f"query schedule {dr, occ, lab} changed the answers")
            trials.append({"query_dense_rows": dr, "query_occupancy": occ, "labels": lab, "ms": round(ms, 4)})
    except BaseException:
        for k, v in before.items():
            set(topo, k, v)
        raise
    best = min(trials, key=lambda r: r["ms"])
    set(topo, "query_dense_rows", best["query_dense_rows"])
    set(topo, "query_occupancy", best["query_occupancy"])
    set(topo, "query_smem_labels_max", smem_max[best["labels"]])
    # then the form for this batch size: a warp or a CTA per query
    nq = s.numel()
    cta_before = get(topo, "query_cta_max")
    forms = {}
    for form, cta_max in (("warp", 0), ("cta", nq)):
        set(topo, "query_cta_max", cta_max)
        forms[form] = _time(torch, lambda: topo.query_batch(metric, s, t, out=out), reps)
        if not torch.equal(ref, out):
            set(topo, "query_cta_max", cta_before)
            raise AssertionError(f"query form {form} changed the answers")
        trials.append({**{k: best[k] for k in ("query_dense_rows", "query_occupancy", "labels")}, "form": form,
                       "ms": round(forms[form], 4)})
    form = min(forms, key=forms.get)
    set(topo, "query_cta_max", max(cta_before, nq) if form == "cta" else min(cta_before, nq - 1))
    chosen = {**{k: best[k] for k in ("query_dense_rows", "query_occupancy", "labels")}, "form": form}
    ms = min(forms.values())
    if form == "warp" and nq > get(topo, "query_cta_max") and top_chains:
        tc_before = get(topo, "query_top_chains")
        tops = {}
        try:
            for tc in top_chains:
                set(topo, "query_top_chains", tc)
                tops[tc] = _time(torch, lambda: topo.query_batch(metric, s, t, out=out), reps)
                if not torch.equal(ref, out):
                    raise AssertionError(f"a top set of {tc} chains changed the answers")
                trials.append({"query_top_chains": tc, "ms": round(tops[tc], 4)})
        except BaseException:
            set(topo, "query_top_chains", tc_before)
            raise
        tc = min(tops, key=tops.get)
        set(topo, "query_top_chains", tc)
        chosen["query_top_chains"] = tc
        ms = tops[tc]
    return {"best": chosen, "ms": round(ms, 4), "trials": trials}


def tune_latency(topo: DeviceTopology, metric: Metric, s_rank, t_rank, dense_rows=(1, 8, 33), wide=(0, 1)) -> dict:
    """The single-query form (a CTA per query): 8 or 16 warps, and its
    row-by-row threshold, timed over one-query calls of the given pairs; the
    fastest is kept (median call)."""
    import torch
    s = torch.as_tensor(np.asarray(s_rank, np.int32)).cuda()
    t = torch.as_tensor(np.asarray(t_rank, np.int32)).cuda()
    out = torch.empty(1, dtype=torch.int64, device="cuda")
    before = {k: get(topo, k) for k in ("query_cta_wide_max", "query_cta_dense_rows")}
    ref, trials = None, []
    try:
        for dr, wd in itertools.product(dense_rows, wide):
            set(topo, "query_cta_dense_rows", dr)
            set(topo, "query_cta_wide_max", 152 if wd else 0)
            res, times = [], []
            for i in range(s.numel()):
                ms = _time(torch, lambda: topo.query_batch(metric, s[i:i + 1], t[i:i + 1], out=out), 1)
                times.append(ms)
                res.append(int(out[0]))
            if ref is None:
                ref = res
            elif res != ref:
                raise AssertionError(f"single-query schedule {(dr, wd)} changed the answers")
            trials.append({"query_cta_dense_rows": dr, "wide": wd, "ms": round(statistics.median(times), 4)})
    except BaseException:
        for k, v in before.items():
            set(topo, k, v)
        raise
    best = min(trials, key=lambda r: r["ms"])
    set(topo, "query_cta_dense_rows", best["query_cta_dense_rows"])
    set(topo, "query_cta_wide_max", 152 if best["wide"] else 0)
    return {"best": best, "trials": trials}


def tune_update(topo: DeviceTopology, metric: Metric, sizes=(1, 10, 100), factors=(0.25, 0.5, 1.0, 2.0),
                seed: int = 0, picks_per_size: int = 5) -> dict:
    """Times raise-and-restore update pairs of each size under sweep budgets
    of `factors` x the default estimate (about a quarter of a full
    customization),
    and with the dense finish at once; keeps the budget and the size from
    which updates go dense at once (`update_dense_min`) with the least total
    time over `sizes`. Each size is timed on `picks_per_size` random arc sets
    and counts with its mean pair, the expected cost: a single arc's update
    is either local (a fraction of a millisecond on the sweep) or reaches
    the top separators (the sweep's budget, then the dense finish), and the
    mix decides. The metric ends as it began."""
    import torch
    rng = np.random.default_rng(seed)
    w0 = metric.w.cpu().numpy().copy()
    default = max(200_000, topo.triangles // 1600)
    before = {k: get(topo, k) for k in ("update_budget_ns", "update_dense_min")}
    picks = {k: [rng.choice(topo.m, size=k, replace=False) for _ in range(picks_per_size)] for k in sizes}
    raises = {k: [w0[ix].astype(np.int64) + 1 + rng.integers(0, 50, k) for ix in picks[k]] for k in sizes}

    def per_size():
        out = {}
        for k in sizes:
            pairs = []
            for idx, up in zip(picks[k], raises[k]):
                total = 0.0
                for val in (up, w0[idx]):
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    topo.update(metric, idx, val)
                    e1.record()
                    torch.cuda.synchronize()
                    total += e0.elapsed_time(e1)
                pairs.append(total)
            out[k] = statistics.fmean(pairs)
        return out

    trials = []
    try:
        set(topo, "update_dense_min", 0)
        sweep = {}
        for f in factors:
            set(topo, "update_budget_ns", max(1, int(default * f)))
            sweep[f] = per_size()
            trials.append({"factor": f, "budget_ns": int(default * f),
                           "ms": {str(k): round(v, 3) for k, v in sweep[f].items()}})
        set(topo, "update_dense_min", 1)
        dense = per_size()
        trials.append({"dense": True, "ms": {str(k): round(v, 3) for k, v in dense.items()}})
    except BaseException:
        for k, v in before.items():
            set(topo, k, v)
        raise
    best = None
    for f in factors:
        for cut in list(sizes) + [0]:  # updates of >= cut arcs go dense at once (0: none)
            total = sum(dense[k] if (cut and k >= cut) else sweep[f][k] for k in sizes)
            if best is None or total < best["ms"]:
                best = {"factor": f, "budget_ns": max(1, int(default * f)), "dense_min": int(cut),
                        "ms": round(total, 3)}
    set(topo, "update_budget_ns", best["budget_ns"])
    set(topo, "update_dense_min", best["dense_min"])
    return {"best": best, "trials": trials}

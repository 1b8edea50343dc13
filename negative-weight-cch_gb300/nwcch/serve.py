"""Serving loop: several customized metrics resident on one GPU, answering a
stream of elimination-tree queries interleaved with arc-update batches.

The reference answers one query per call on one metric (python/cch_nb.py:
577-615, driven by python/run_nb.py:127-141) and applies updates through
CCH.update_edges (python/cch.py:349-402). This module keeps the same
per-request semantics and adds the serving layer around the device calls:

* Metrics are registered with their weights and admitted to the device while
  their buffers fit a memory budget; an idle metric (no pending work) is
  evicted, least recently used first, to admit another. Its current weights
  stay on the host and it is customized again on its next admission.
* Every registered metric has a slot: a worker thread with its own CUDA
  stream. Requests of a metric are served in arrival order. Whenever the slot
  is free it takes every query that arrived meanwhile (up to `max_batch`,
  stopping at the next update) as one batched launch: continuous batching,
  so requests that arrive while a batch runs join the next one, and the slots
  of different metrics overlap on the device.
* An update batch is applied in place by the partial re-customization; the
  queries behind it see the updated metric, those before it the old one.

So the answer of a query depends only on the metric, on the updates of that
metric that arrived before it and on (s, t), never on what else was in the
mix; the `version` of an answer is the number of those updates.

Queries travel in blocks (numpy arrays of s, t and arrival times) so that an
open-loop generator can offer a million queries a second from one thread.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from .device import DeviceTopology, Metric


class QueryBlock:
    """Queries of one metric submitted together. Filled in as answered:
    result (int64 distance, INT64_MAX = unreachable), done (perf_counter
    time the answer was on the host), version."""

    def __init__(self, key, s, t, arrival):
        self.key = key
        self.s = np.ascontiguousarray(s, np.int32).ravel()
        self.t = np.ascontiguousarray(t, np.int32).ravel()
        n = self.s.size
        if self.t.size != n:
            raise ValueError("s and t differ in length")
        self.arrival = np.broadcast_to(np.asarray(arrival, np.float64), (n,)).copy()
        self.result = np.full(n, -1, np.int64)
        self.done = np.zeros(n, np.float64)
        self.version = np.full(n, -1, np.int32)
        self.error: str | None = None
        self._left = n
        self._event = threading.Event()
        if n == 0:
            self._event.set()

    def __len__(self) -> int:
        return self.s.size

    def wait(self, timeout: float | None = None) -> bool:
        return self._event.wait(timeout)

    def _answered(self, count: int) -> None:
        self._left -= count
        if self._left <= 0:
            self._event.set()

    @property
    def latency(self) -> np.ndarray:
        return self.done - self.arrival


@dataclass
class UpdateRequest:
    key: object
    edge_idx: np.ndarray
    new_w: np.ndarray
    arrival: float = 0.0
    done: float = 0.0
    evaluated: int = -1        # arcs re-evaluated (CCH.update_edges' return value)
    version: int = -1          # updates of this metric applied, this one included
    negative_cycle: bool = False  # a changed arc closed a negative cycle
    error: str | None = None
    _event: threading.Event = field(default_factory=threading.Event, repr=False)

    def wait(self, timeout: float | None = None) -> bool:
        return self._event.wait(timeout)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class _Slot:
    """One registered metric: host weights, device state when resident."""

    def __init__(self, key, w: np.ndarray):
        self.key = key
        self.w = np.ascontiguousarray(w, np.int32).copy()  # current weights (updates applied)
        self.metric: Metric | None = None
        self.queue: collections.deque = collections.deque()  # [block, start] or UpdateRequest
        self.pending_queries = 0
        self.version = 0
        self.busy = False
        self.last_use = 0.0
        self.thread: threading.Thread | None = None
        self.stream = None
        self.bufs = None


class ServingLoop:
    """Request loop over one DeviceTopology.

    memory_budget: bytes of device memory the resident metrics may hold
    (default: 80% of the free device memory at construction). max_batch:
    most queries per launch. method: "supernodal" (batched kernel) or
    "plain" (one ancestor at a time)."""

    def __init__(self, topo: DeviceTopology, memory_budget: int | None = None, max_batch: int = 1 << 16,
                 method: str = "supernodal"):
        import torch
        self.torch = torch
        self.topo = topo
        self.method = method
        self.max_batch = int(max_batch)
        if memory_budget is None:
            free, _ = torch.cuda.mem_get_info()
            memory_budget = int(free * 0.8)
        self.memory_budget = int(memory_budget)
        self.metric_bytes = topo.m_plus * 8 + topo.m * 4
        self.batch_bytes = self.max_batch * (4 + 4 + 8)
        self._slots: dict[object, _Slot] = {}
        self._mu = threading.Condition()
        self._resident = 0
        self._closed = False
        self.batches = 0
        self.batched_queries = 0
        self.admissions = 0
        self.evictions = 0

    # ------------------------------------------------------------ metrics
    def cost(self) -> int:
        """Device bytes one resident metric holds."""
        return self.metric_bytes + self.batch_bytes

    def add_metric(self, key, w) -> None:
        """Registers a metric (int32 weights of the topology's original arcs);
        it is customized on the device when first admitted."""
        w = np.asarray(w)
        if w.size != self.topo.m:
            raise ValueError(f"expected {self.topo.m} weights, got {w.size}")
        if self.cost() > self.memory_budget:
            raise MemoryError(f"one metric needs {self.cost()} bytes, budget {self.memory_budget}")
        with self._mu:
            if key in self._slots:
                raise KeyError(f"metric {key!r} already registered")
            slot = _Slot(key, w)
            self._slots[key] = slot
            slot.thread = threading.Thread(target=self._worker, args=(slot,), daemon=True,
                                           name=f"nwcch-serve-{key}")
            slot.thread.start()

    def resident(self) -> list:
        with self._mu:
            return [k for k, s in self._slots.items() if s.metric is not None]

    def _admit(self, slot: _Slot) -> bool:
        """With self._mu held: makes room for `slot` (evicting idle metrics,
        least recently used first). False if nothing can be evicted yet."""
        need = self.cost()
        while self._resident + need > self.memory_budget:
            idle = [s for s in self._slots.values()
                    if s is not slot and s.metric is not None and not s.busy and not s.queue]
            if not idle:
                return False
            victim = min(idle, key=lambda s: s.last_use)
            victim.metric = None
            victim.bufs = None
            self._resident -= need
            self.evictions += 1
        self._resident += need
        self.admissions += 1
        return True

    # ------------------------------------------------------------ requests
    def submit_queries(self, key, s_rank, t_rank, arrival=None) -> QueryBlock:
        """Queries (rank pairs) on one metric; `arrival` (perf_counter
        seconds, scalar or per query) defaults to now."""
        blk = QueryBlock(key, s_rank, t_rank, time.perf_counter() if arrival is None else arrival)
        if len(blk):
            n = self.topo.n
            if blk.s.min() < 0 or blk.s.max() >= n or blk.t.min() < 0 or blk.t.max() >= n:
                raise ValueError("rank out of range")
            self._enqueue(key, blk)
        return blk

    def submit_query(self, key, s_rank: int, t_rank: int) -> QueryBlock:
        return self.submit_queries(key, [s_rank], [t_rank])

    def submit_update(self, key, edge_idx, new_w, arrival: float | None = None) -> UpdateRequest:
        idx = np.ascontiguousarray(edge_idx, np.int64).ravel()
        val = np.ascontiguousarray(new_w, np.int64).ravel()
        if idx.size != val.size:
            raise ValueError("edge_idx and new_w differ in length")
        if idx.size and (idx.min() < 0 or idx.max() >= self.topo.m):
            raise ValueError("original arc id out of range")
        r = UpdateRequest(key, idx, val, arrival=time.perf_counter() if arrival is None else arrival)
        self._enqueue(key, r)
        return r

    def _enqueue(self, key, item) -> None:
        with self._mu:
            if self._closed:
                raise RuntimeError("serving loop is closed")
            slot = self._slots.get(key)
            if slot is None:
                raise KeyError(f"unknown metric {key!r}")
            if isinstance(item, QueryBlock):
                slot.queue.append([item, 0])
                slot.pending_queries += len(item)
            else:
                slot.queue.append(item)
            self._mu.notify_all()

    def close(self) -> None:
        with self._mu:
            self._closed = True
            self._mu.notify_all()
        for s in self._slots.values():
            if s.thread is not None:
                s.thread.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------ worker
    def _take(self, slot: _Slot):
        """With self._mu held: the next unit of work of `slot`: an update, or
        up to max_batch queries as (block, start, end) pieces."""
        head = slot.queue[0]
        if isinstance(head, UpdateRequest):
            return slot.queue.popleft()
        pieces, n = [], 0
        while slot.queue and not isinstance(slot.queue[0], UpdateRequest) and n < self.max_batch:
            entry = slot.queue[0]
            blk, start = entry
            end = min(len(blk), start + self.max_batch - n)
            pieces.append((blk, start, end))
            n += end - start
            if end == len(blk):
                slot.queue.popleft()
            else:
                entry[1] = end
        slot.pending_queries -= n
        return pieces

    def _worker(self, slot: _Slot) -> None:
        torch = self.torch
        slot.stream = torch.cuda.Stream()
        while True:
            with self._mu:
                while not self._closed and (not slot.queue or (slot.metric is None and not self._admit(slot))):
                    self._mu.wait(0.05)
                if not slot.queue:
                    return  # closed and drained
                slot.busy = True
                work = self._take(slot)
            try:
                if slot.metric is None:
                    try:
                        self._materialize(slot)
                    except Exception:
                        with self._mu:  # give the admitted room back
                            slot.metric = None
                            slot.bufs = None
                            self._resident -= self.cost()
                        raise
                with torch.cuda.stream(slot.stream):
                    if isinstance(work, UpdateRequest):
                        self._apply_update(slot, work)
                    else:
                        self._run_queries(slot, work)
            except Exception as e:  # reported on every request of the unit
                msg = f"{type(e).__name__}: {e}"
                now = time.perf_counter()
                if isinstance(work, UpdateRequest):
                    work.error, work.done = msg, now
                    work._event.set()
                else:
                    for blk, a, b in work:
                        blk.error = msg
                        blk.done[a:b] = now
                        blk._answered(b - a)
            finally:
                with self._mu:
                    slot.busy = False
                    slot.last_use = time.perf_counter()
                    self._mu.notify_all()

    def _materialize(self, slot: _Slot) -> None:
        """Customizes an admitted metric. Its buffers come from the default
        stream's pool, so that they return to a pool every slot draws on when
        the metric is evicted (only ever while its slot is idle)."""
        torch = self.torch
        with torch.cuda.stream(torch.cuda.default_stream()):
            metric = self.topo.customize(slot.w, "int32")
            B = self.max_batch
            bufs = dict(
                s_host=torch.empty(B, dtype=torch.int32).pin_memory(),
                t_host=torch.empty(B, dtype=torch.int32).pin_memory(),
                d_host=torch.empty(B, dtype=torch.int64).pin_memory(),
                s_dev=torch.empty(B, dtype=torch.int32, device="cuda"),
                t_dev=torch.empty(B, dtype=torch.int32, device="cuda"),
                d_dev=torch.empty(B, dtype=torch.int64, device="cuda"))
            torch.cuda.default_stream().synchronize()
        slot.metric, slot.bufs = metric, bufs

    def _run_queries(self, slot: _Slot, pieces) -> None:
        b = slot.bufs
        s_np = b["s_host"].numpy()
        t_np = b["t_host"].numpy()
        n = 0
        for blk, a, e in pieces:
            s_np[n:n + e - a] = blk.s[a:e]
            t_np[n:n + e - a] = blk.t[a:e]
            n += e - a
        b["s_dev"][:n].copy_(b["s_host"][:n], non_blocking=True)
        b["t_dev"][:n].copy_(b["t_host"][:n], non_blocking=True)
        self.topo.query_batch(slot.metric, b["s_dev"][:n], b["t_dev"][:n], method=self.method,
                              out=b["d_dev"][:n])
        b["d_host"][:n].copy_(b["d_dev"][:n], non_blocking=True)
        slot.stream.synchronize()
        d = b["d_host"].numpy()
        now = time.perf_counter()
        o = 0
        for blk, a, e in pieces:
            blk.result[a:e] = d[o:o + e - a]
            blk.version[a:e] = slot.version
            blk.done[a:e] = now
            o += e - a
            blk._answered(e - a)
        with self._mu:
            self.batches += 1
            self.batched_queries += n

    def _apply_update(self, slot: _Slot, r: UpdateRequest) -> None:
        ev = self.topo.update(slot.metric, r.edge_idx, r.new_w)
        slot.w[r.edge_idx] = r.new_w.astype(np.int32)
        slot.stream.synchronize()
        slot.version += 1
        r.evaluated = int(ev)
        r.negative_cycle = slot.metric.stats.get("changed_negative", 0) > 0
        r.version = slot.version
        r.done = time.perf_counter()
        r._event.set()


# ---------------------------------------------------------------- traces

@dataclass
class Trace:
    """Open-loop workload: query arrivals (seconds from the start, metric
    index into `keys`, source and target ranks) and update batches
    (seconds, metric index, original arc ids, new weights)."""
    keys: list
    q_time: np.ndarray
    q_metric: np.ndarray
    q_s: np.ndarray
    q_t: np.ndarray
    updates: list  # [(time, metric index, edge_idx, new_w)]

    @property
    def queries(self) -> int:
        return int(self.q_time.size)


@dataclass
class TraceResult:
    trace: Trace
    result: np.ndarray    # per query, in trace order
    latency: np.ndarray   # seconds from scheduled arrival to answer on the host
    version: np.ndarray
    done: np.ndarray
    start: float
    updates: list          # UpdateRequest per trace update, in trace order
    errors: list


def poisson_trace(topo: DeviceTopology, keys: list, rate: float, duration: float, update_every: float = 0.0,
                  update_sizes=(1, 10, 100, 1000), weights: dict | None = None, L: np.ndarray | None = None,
                  seed: int = 0) -> Trace:
    """Poisson query arrivals at `rate` per second for `duration` seconds
    (uniform s, t ranks and uniform metric), plus an update batch every
    `update_every` seconds on average (Poisson; size drawn from
    update_sizes). With `weights` (key -> int32 weights, advanced in place)
    and L (per-arc lengths of the initial weights), an update gives an arc a
    new length L' uniform in [1, 2L], w' = w - (current length) + L': lengths
    change, heights do not, so every metric stays free of negative cycles."""
    rng = np.random.default_rng(seed)
    nq = int(rng.poisson(rate * duration))
    q_time = np.sort(rng.uniform(0, duration, nq))
    q_s = rng.integers(0, topo.n, nq).astype(np.int32)
    q_t = rng.integers(0, topo.n, nq).astype(np.int32)
    q_metric = rng.integers(0, len(keys), nq).astype(np.int32)
    updates = []
    lengths = {}
    if update_every > 0:
        nu = int(rng.poisson(duration / update_every))
        for tu in np.sort(rng.uniform(0, duration, nu)):
            j = int(rng.integers(len(keys)))
            size = int(update_sizes[int(rng.integers(len(update_sizes)))])
            idx = rng.choice(topo.m, size=size, replace=False).astype(np.int64)
            if weights is not None and L is not None:
                w = weights[keys[j]]
                cur = lengths.setdefault(j, np.asarray(L, np.int64).copy())
                Li = np.asarray(L, np.int64)[idx]
                new_len = rng.integers(1, 2 * Li + 1)
                val = w[idx].astype(np.int64) - cur[idx] + new_len
                cur[idx] = new_len
                w[idx] = val
            else:
                val = rng.integers(1, 1000, size).astype(np.int64)
            updates.append((float(tu), j, idx, val))
    return Trace(list(keys), q_time, q_metric, q_s, q_t, updates)


def run_trace(loop: ServingLoop, trace: Trace, step: float = 1e-4, timeout: float = 600.0) -> TraceResult:
    """Offers `trace` to `loop` in real time (open loop: arrivals never wait
    for answers). Every `step` seconds the requests whose arrival time has
    passed are submitted, queries of one metric as one block, in time order
    with the updates; latency counts from the scheduled arrival."""
    keys = trace.keys
    upd_t = np.array([u[0] for u in trace.updates], np.float64)
    blocks = []  # (query indices, QueryBlock)
    ureqs = []
    qi = ui = 0
    nq = trace.queries
    t0 = time.perf_counter()
    while qi < nq or ui < len(trace.updates):
        now = time.perf_counter() - t0
        # events due by now, in time order: queries up to the next due update,
        # then that update, and so on
        while True:
            next_u = upd_t[ui] if ui < len(upd_t) else np.inf
            limit = min(now, next_u)
            qe = int(np.searchsorted(trace.q_time, limit, side="right" if next_u > now else "left"))
            if qe > qi:
                sl = np.arange(qi, qe)
                mk = trace.q_metric[qi:qe]
                for j in np.unique(mk):
                    sel = sl[mk == j]
                    blocks.append((sel, loop.submit_queries(keys[j], trace.q_s[sel], trace.q_t[sel],
                                                            arrival=t0 + trace.q_time[sel])))
                qi = qe
            if next_u <= now:
                tu, j, idx, val = trace.updates[ui]
                ureqs.append(loop.submit_update(keys[j], idx, val, arrival=t0 + tu))
                ui += 1
                continue
            break
        nxt = min(trace.q_time[qi] if qi < nq else np.inf, upd_t[ui] if ui < len(upd_t) else np.inf)
        if np.isfinite(nxt):
            dt = t0 + nxt - time.perf_counter()
            if dt > 0:
                time.sleep(min(dt, step))
    deadline = time.perf_counter() + timeout
    for _, blk in blocks:
        if not blk.wait(max(0.0, deadline - time.perf_counter())):
            raise TimeoutError("serving trace did not finish")
    for r in ureqs:
        if not r.wait(max(0.0, deadline - time.perf_counter())):
            raise TimeoutError("serving trace did not finish")
    result = np.empty(nq, np.int64)
    latency = np.empty(nq, np.float64)
    version = np.empty(nq, np.int32)
    done = np.empty(nq, np.float64)
    errors = []
    for sel, blk in blocks:
        result[sel] = blk.result
        latency[sel] = blk.latency
        version[sel] = blk.version
        done[sel] = blk.done
        if blk.error:
            errors.append(blk.error)
    errors += [r.error for r in ureqs if r.error]
    return TraceResult(trace, result, latency, version, done, t0, ureqs, errors)


def summarize(res: TraceResult) -> dict:
    """Latency percentiles (ms) and throughput of an answered trace."""
    out = {"queries": res.trace.queries, "updates": len(res.updates), "errors": len(res.errors)}
    if res.trace.queries:
        lat = res.latency * 1000
        span = res.done.max() - (res.start + res.trace.q_time.min())
        out.update(p50_ms=round(float(np.percentile(lat, 50)), 4), p99_ms=round(float(np.percentile(lat, 99)), 4),
                   mean_ms=round(float(lat.mean()), 4),
                   queries_per_s=round(res.trace.queries / span, 1) if span > 0 else None)
    if res.updates:
        ul = np.array([r.latency for r in res.updates]) * 1000
        out.update(update_p50_ms=round(float(np.percentile(ul, 50)), 4),
                   update_p99_ms=round(float(np.percentile(ul, 99)), 4))
    return out

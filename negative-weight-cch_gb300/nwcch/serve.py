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
* Every resident metric has a slot: a worker thread with its own CUDA stream.
  Requests of a metric are served in arrival order. Whenever the slot is free
  it takes every query that arrived meanwhile (up to `max_batch`, stopping at
  the next update) as one batched launch: continuous batching, so requests
  that arrive while a batch runs join the next one, and the slots of
  different metrics overlap on the device.
* An update batch is applied in place by the partial re-customization; the
  queries behind it see the updated metric, those before it the old one.

So the answer of a query depends only on the metric, on the updates of that
metric that arrived before it and on (s, t), never on what else was in the
mix; `Request.version` records the number of those updates.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .device import DeviceTopology, Metric


@dataclass
class Request:
    kind: str                 # "query" or "update"
    key: object               # metric key
    s: int = -1               # query: source rank
    t: int = -1               # query: target rank
    edge_idx: np.ndarray | None = None   # update: original arc ids
    new_w: np.ndarray | None = None      # update: new integer weights
    arrival: float = 0.0      # perf_counter() time the request arrived
    done: float = 0.0         # perf_counter() time its result was on the host
    result: int | None = None  # query: distance (INT64_MAX = unreachable); update: arcs evaluated
    version: int = -1         # updates of this metric applied before it
    negative_cycle: bool = False  # update: an arc it changed closed a negative cycle
    error: str | None = None
    event: threading.Event = field(default_factory=threading.Event, repr=False)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class _Slot:
    """One registered metric: host weights, device state when resident."""

    def __init__(self, key, w: np.ndarray):
        self.key = key
        self.w = np.ascontiguousarray(w, np.int32).copy()  # current weights (updates applied)
        self.metric: Metric | None = None
        self.queue: collections.deque[Request] = collections.deque()
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
    def add_metric(self, key, w) -> None:
        """Registers a metric (int32 weights of the topology's original arcs);
        it is customized on the device when first admitted."""
        w = np.asarray(w)
        if w.size != self.topo.m:
            raise ValueError(f"expected {self.topo.m} weights, got {w.size}")
        if self._cost() > self.memory_budget:
            raise MemoryError(f"one metric needs {self._cost()} bytes, budget {self.memory_budget}")
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

    def _cost(self) -> int:
        return self.metric_bytes + self.batch_bytes

    def _admit(self, slot: _Slot) -> bool:
        """With self._mu held: makes room for `slot` (evicting idle metrics,
        least recently used first). False if nothing can be evicted yet."""
        need = self._cost()
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
    def submit_query(self, key, s_rank: int, t_rank: int) -> Request:
        r = Request("query", key, s=int(s_rank), t=int(t_rank))
        self._submit(r)
        return r

    def submit_update(self, key, edge_idx, new_w) -> Request:
        idx = np.ascontiguousarray(edge_idx, np.int64).ravel()
        val = np.ascontiguousarray(new_w, np.int64).ravel()
        if idx.size != val.size:
            raise ValueError("edge_idx and new_w differ in length")
        if idx.size and (idx.min() < 0 or idx.max() >= self.topo.m):
            raise ValueError("original arc id out of range")
        r = Request("update", key, edge_idx=idx, new_w=val)
        self._submit(r)
        return r

    def _submit(self, r: Request) -> None:
        with self._mu:
            if self._closed:
                raise RuntimeError("serving loop is closed")
            slot = self._slots.get(r.key)
            if slot is None:
                raise KeyError(f"unknown metric {r.key!r}")
            r.arrival = time.perf_counter()
            slot.queue.append(r)
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
    def _worker(self, slot: _Slot) -> None:
        torch = self.torch
        slot.stream = torch.cuda.Stream()
        while True:
            with self._mu:
                while not self._closed and (not slot.queue or (slot.metric is None and not self._admit(slot))):
                    self._mu.wait(0.05)
                if self._closed and not slot.queue:
                    return
                slot.busy = True
                head = slot.queue[0]
                if head.kind == "update":
                    work = [slot.queue.popleft()]
                else:
                    work = []
                    while slot.queue and slot.queue[0].kind == "query" and len(work) < self.max_batch:
                        work.append(slot.queue.popleft())
            try:
                if slot.metric is None:
                    try:
                        self._materialize(slot)
                    except Exception:
                        with self._mu:  # give the admitted room back
                            slot.metric = None
                            slot.bufs = None
                            self._resident -= self._cost()
                        raise
                with torch.cuda.stream(slot.stream):
                    if work[0].kind == "update":
                        self._apply_update(slot, work[0])
                    else:
                        self._run_queries(slot, work)
            except Exception as e:  # report on every request of the batch
                now = time.perf_counter()
                for r in work:
                    r.error = f"{type(e).__name__}: {e}"
                    r.done = now
                    r.event.set()
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
            self._customize(slot)

    def _customize(self, slot: _Slot) -> None:
        torch = self.torch
        slot.metric = self.topo.customize(slot.w, "int32")
        B = self.max_batch
        slot.bufs = dict(
            s_host=torch.empty(B, dtype=torch.int32).pin_memory(),
            t_host=torch.empty(B, dtype=torch.int32).pin_memory(),
            d_host=torch.empty(B, dtype=torch.int64).pin_memory(),
            s_dev=torch.empty(B, dtype=torch.int32, device="cuda"),
            t_dev=torch.empty(B, dtype=torch.int32, device="cuda"),
            d_dev=torch.empty(B, dtype=torch.int64, device="cuda"))

    def _run_queries(self, slot: _Slot, work: list[Request]) -> None:
        b = slot.bufs
        n = len(work)
        s_np = b["s_host"].numpy()
        t_np = b["t_host"].numpy()
        for i, r in enumerate(work):
            s_np[i] = r.s
            t_np[i] = r.t
        b["s_dev"][:n].copy_(b["s_host"][:n], non_blocking=True)
        b["t_dev"][:n].copy_(b["t_host"][:n], non_blocking=True)
        self.topo.query_batch(slot.metric, b["s_dev"][:n], b["t_dev"][:n], method=self.method,
                              out=b["d_dev"][:n])
        b["d_host"][:n].copy_(b["d_dev"][:n], non_blocking=True)
        slot.stream.synchronize()
        d = b["d_host"].numpy()[:n]
        now = time.perf_counter()
        for i, r in enumerate(work):
            r.result = int(d[i])
            r.version = slot.version
            r.done = now
            r.event.set()
        with self._mu:
            self.batches += 1
            self.batched_queries += n

    def _apply_update(self, slot: _Slot, r: Request) -> None:
        ev = self.topo.update(slot.metric, r.edge_idx, r.new_w)
        slot.w[r.edge_idx] = r.new_w.astype(np.int32)
        slot.stream.synchronize()
        r.result = int(ev)
        r.negative_cycle = slot.metric.stats.get("changed_negative", 0) > 0
        slot.version += 1
        r.version = slot.version
        r.done = time.perf_counter()
        r.event.set()

    # ------------------------------------------------------------ traces
    def run_trace(self, trace: list[tuple[float, Request]], timeout: float = 300.0) -> list[Request]:
        """Submits each (offset seconds, request template) at its offset from
        now (open loop: arrivals do not wait for answers) and returns the
        requests once all are answered."""
        out = []
        t0 = time.perf_counter()
        for off, tmpl in trace:
            while True:
                dt = t0 + off - time.perf_counter()
                if dt <= 0:
                    break
                if dt > 2e-4:
                    time.sleep(dt - 1e-4)
            if tmpl.kind == "query":
                out.append(self.submit_query(tmpl.key, tmpl.s, tmpl.t))
            else:
                out.append(self.submit_update(tmpl.key, tmpl.edge_idx, tmpl.new_w))
        deadline = time.perf_counter() + timeout
        for r in out:
            if not r.event.wait(max(0.0, deadline - time.perf_counter())):
                raise TimeoutError("serving trace did not finish")
        return out


def poisson_trace(topo: DeviceTopology, keys: list, rate: float, duration: float, update_every: float,
                  update_sizes=(1, 10, 100, 1000), weights: dict | None = None, L: np.ndarray | None = None,
                  seed: int = 0) -> list[tuple[float, Request]]:
    """Open-loop trace: Poisson query arrivals at `rate` per second for
    `duration` seconds (uniform s, t ranks and uniform metric), plus an
    update batch every `update_every` seconds on average (Poisson; size
    drawn from update_sizes). With `weights` (key -> int32 weights, advanced
    in place) and L (per-arc lengths), an update sets w' = w + L' - L for
    L' uniform in [1, 2L]: lengths change, heights do not, so every metric
    stays free of negative cycles."""
    rng = np.random.default_rng(seed)
    n = topo.n
    trace = []
    nq = rng.poisson(rate * duration)
    tq = np.sort(rng.uniform(0, duration, nq))
    s = rng.integers(0, n, nq)
    t = rng.integers(0, n, nq)
    k = rng.integers(0, len(keys), nq)
    for i in range(nq):
        trace.append((float(tq[i]), Request("query", keys[k[i]], s=int(s[i]), t=int(t[i]))))
    if update_every > 0:
        nu = rng.poisson(duration / update_every)
        tu = np.sort(rng.uniform(0, duration, nu))
        for i in range(nu):
            key = keys[int(rng.integers(len(keys)))]
            size = int(update_sizes[int(rng.integers(len(update_sizes)))])
            idx = rng.choice(topo.m, size=size, replace=False).astype(np.int64)
            if weights is not None and L is not None:
                w = weights[key]
                Li = L[idx].astype(np.int64)
                val = w[idx].astype(np.int64) + rng.integers(1, 2 * Li + 1) - Li
                w[idx] = val
            else:
                val = rng.integers(1, 1000, size).astype(np.int64)
            trace.append((float(tu[i]), Request("update", key, edge_idx=idx, new_w=val)))
    trace.sort(key=lambda x: x[0])
    return trace


def summarize(reqs: list[Request]) -> dict:
    """Latency percentiles (ms) and throughput of an answered trace."""
    q = [r for r in reqs if r.kind == "query" and r.error is None]
    u = [r for r in reqs if r.kind == "update" and r.error is None]
    errors = sum(r.error is not None for r in reqs)
    out = {"queries": len(q), "updates": len(u), "errors": errors}
    if q:
        lat = np.array([r.latency for r in q]) * 1000
        span = max(r.done for r in q) - min(r.arrival for r in q)
        out.update(p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                   mean_ms=float(lat.mean()), queries_per_s=len(q) / span if span > 0 else None)
    if u:
        lat = np.array([r.latency for r in u]) * 1000
        out.update(update_p50_ms=float(np.percentile(lat, 50)), update_p99_ms=float(np.percentile(lat, 99)))
    return out


INF = _lib.INF64

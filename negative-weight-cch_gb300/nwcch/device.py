"""Device-resident topology and metrics over the libnwcch C ABI.

PyTorch provides the device buffers and the current CUDA stream; every kernel
is libnwcch's own sm_103a code. There is no CPU fallback: without a CUDA
device (or without the built library) every call raises.
"""
from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib

P, I64, I32 = C.c_void_p, C.c_int64, C.c_int32
PP = C.POINTER(C.c_void_p)
PI64 = C.POINTER(C.c_int64)

for _name, _args in {
    "nwcch_topology_create": [I64, P, P, P, I64, P, P, PP],
    "nwcch_topology_destroy": [P],
    "nwcch_topology_info": [P, P, I64],
    "nwcch_topology_export": [P, C.c_int, P, I64],
    "nwcch_check": [P, P],
    "nwcch_customize": [P, P, P, P, P],
    "nwcch_customize_async": [P, P, P, P, P],
    "nwcch_customize_i64": [P, P, P, P, P],
    "nwcch_customize_i64_async": [P, P, P, P, P],
    "nwcch_customize_plain": [P, P, P, P, P],
    "nwcch_customize_plain_async": [P, P, P, P, P],
    "nwcch_negative_cycle_arcs": [P, P, P, PI64, P],
    "nwcch_negative_cycle_arcs_i64": [P, P, P, PI64, P],
    "nwcch_negative_cycle_arcs_async": [P, P, P, P, P],
    "nwcch_customize_batch": [P, I64, P, P, P, P],
    "nwcch_customize_batch_async": [P, I64, P, P, P, P],
    "nwcch_negative_cycle_arcs_batch_async": [P, I64, P, P, P, P],
    "nwcch_query_batch_noalloc": [P, P, P, P, P, I64, P, P],
    "nwcch_query_batch_async": [P, P, P, P, P, I64, P, P],
    "nwcch_query_batch_plain": [P, P, P, P, P, I64, P, P],
    "nwcch_negative_loops": [P, P, PI64, P],
    "nwcch_update": [P, P, P, P, P, P, I64, P, P, P],
    "nwcch_update_i64": [P, P, P, P, P, P, I64, P, P, P],
    "nwcch_query_batch": [P, P, P, P, P, I64, P, P],
    "nwcch_query_batch_i64": [P, P, P, P, P, I64, P, P],
    "nwcch_potential": [P, P, P, P, P],
    "nwcch_query_paths": [P, P, P, P, P, I64, P, P, P, I64, PI64, P],
    "nwcch_query_paths_i64": [P, P, P, P, P, I64, P, P, P, I64, PI64, P],
    "nwcch_potential_i64": [P, P, P, P, P],
}.items():
    _lib.register(_name, _args)

SATURATED = 1


class SaturationWarning(RuntimeWarning):
    """Some customized values were clamped to the storage range."""


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("nwcch device calls need a CUDA device (no CPU fallback)")
    return torch


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _status(code: int, where: str) -> bool:
    """True if the call saturated; raises on errors."""
    if code == SATURATED:
        return True
    _lib.check(code, where)
    return False


def parent_from_rows(first, head):
    """parent[x] = lowest upper neighbour of x (first entry of its sorted row)."""
    first = np.asarray(first, np.int64)
    n = first.size - 1
    deg = np.diff(first)
    parent = np.full(n, -1, np.int64)
    has = deg > 0
    parent[has] = np.asarray(head)[first[:-1][has]]
    return parent


@dataclass
class Metric:
    """One customized metric resident on the device."""
    topo: "DeviceTopology"
    w: object        # torch int32 [m], current original weights
    up: object       # torch int32/int64 [m+]
    dn: object
    saturated: bool = False
    last_changed: object = None
    stats: dict = field(default_factory=dict)

    @property
    def storage(self) -> str:
        return "int64" if self.up.element_size() == 8 else "int32"

    def to_numpy(self):
        """(up, dn) as int64 numpy arrays with INT64_MAX for "no path"."""
        inf_in = _lib.INF32 if self.storage == "int32" else _lib.INF64
        out = []
        for t in (self.up, self.dn):
            a = t.cpu().numpy().astype(np.int64)
            a[a == inf_in] = _lib.INF64
            out.append(a)
        return tuple(out)

    def to_reference(self):
        """(upw, dnw) in the reference's convention: float64 with inf."""
        out = []
        for a in self.to_numpy():
            f = a.astype(np.float64)
            f[a == _lib.INF64] = np.inf
            out.append(f)
        return tuple(out)


@dataclass
class MetricBatch:
    """K customized metrics of one topology, metric-major on the device."""
    topo: "DeviceTopology"
    w: object        # torch int32 [K, m]
    up: object       # torch int32 [K, m+]
    dn: object
    saturated: bool = False

    def __len__(self) -> int:
        return int(self.up.shape[0])

    def metric(self, k: int) -> Metric:
        """Metric k as a view: queries and updates on it act on the batch."""
        return Metric(self.topo, self.w[k], self.up[k], self.dn[k], saturated=self.saturated)


class DeviceTopology:
    """Validated, extended and uploaded contracted graph (one handle)."""

    def __init__(self, n, first, head, parent, e_arc, e_up):
        self._torch = _torch()
        lib = _lib.lib()
        self.n = int(n)
        first = np.ascontiguousarray(first, np.int64)
        head = np.ascontiguousarray(head, np.int32)
        parent = np.ascontiguousarray(parent if parent is not None else parent_from_rows(first, head), np.int32)
        e_arc = np.ascontiguousarray(e_arc, np.int64)
        e_up = np.ascontiguousarray(e_up, np.int8)
        h = C.c_void_p()
        self._torch.cuda.init()
        _lib.check(lib.nwcch_topology_create(self.n, _lib.ptr(first), _lib.ptr(head), _lib.ptr(parent), e_arc.size,
                                             _lib.ptr(e_arc), _lib.ptr(e_up), C.byref(h)), "topology_create")
        self._h = h
        self.refresh_info()

    def refresh_info(self):
        """Re-reads the handle's figures (the plan's change when re-planned)."""
        info = np.zeros(16, np.int64)
        _lib.check(_lib.lib().nwcch_topology_info(self.handle, _lib.ptr(info), 16), "topology_info")
        (self.n, self.m_plus, self.m, self.triangles, self.levels, self.depth, self.max_row,
         self.device_bytes, self.supernodes, self.sn_levels, self.sn_launches,
         self.rel_entries, self.chain_level, self.chain_phases, self.chain_from, _) = (int(v) for v in info)

    def last_query_launches(self) -> int:
        """Kernels the latest batched-query call on this handle enqueued."""
        info = np.zeros(16, np.int64)
        _lib.check(_lib.lib().nwcch_topology_info(self.handle, _lib.ptr(info), 16), "topology_info")
        return int(info[15])

    # name -> (key, dtype, length from the handle's figures)
    _ARRAYS = {"tail": (0, np.int32), "depth": (1, np.int32), "hdep": (2, np.int32), "doff": (3, np.int64),
               "darc": (4, np.int32), "level": (5, np.int32), "aeoff": (6, np.int64), "aeidx": (7, np.int32),
               "level_verts": (8, np.int32), "loops": (9, np.int32), "level_off": (10, np.int64),
               "level_arcs": (11, np.int64), "level_tri": (12, np.int64), "level_maxdeg": (13, np.int32)}

    def export(self, name: str) -> np.ndarray:
        """A derived array of the handle (built on the device from first,
        head, parent and e_arc), copied to host memory."""
        key, dt = self._ARRAYS[name]
        if name in ("aeidx", "loops"):
            aeoff = self.export("aeoff")
            length = int(aeoff[-1]) if name == "aeidx" else self.m - int(aeoff[-1])
        else:
            length = {"tail": self.m_plus, "depth": self.n, "hdep": self.m_plus, "doff": self.n + 1,
                      "darc": self.m_plus, "level": self.n, "aeoff": self.m_plus + 1, "level_verts": self.n,
                      "level_off": self.levels + 1, "level_arcs": self.levels + 1, "level_tri": self.levels,
                      "level_maxdeg": self.levels}[name]
        out = np.empty(max(length, 1), dt)
        _lib.check(_lib.lib().nwcch_topology_export(self.handle, key, _lib.ptr(out), length), "topology_export")
        return out[:length]

    @classmethod
    def from_dict(cls, t: dict) -> "DeviceTopology":
        return cls(t["n"], t["first"], t["head"], t.get("parent"), t["e_arc"], t["e_up"])

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("topology is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.lib().nwcch_topology_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ helpers
    def weights(self, w):
        """int32 device tensor of original weights (copied from host if needed)."""
        torch = self._torch
        if isinstance(w, torch.Tensor):
            t = w.to(device="cuda", dtype=torch.int32)
        else:
            a = np.asarray(w)
            if a.dtype.kind == "f":
                if not np.all(np.isfinite(a)) or not np.array_equal(a, np.rint(a)):
                    raise ValueError("weights must be integral")
            a = a.astype(np.int64)
            if a.size and (a.max() >= _lib.INF32 or a.min() < -_lib.INF32):
                raise ValueError("weights must fit int32 (and differ from INT32_MAX)")
            t = torch.from_numpy(a.astype(np.int32)).to("cuda")
        if t.numel() != self.m:
            raise ValueError(f"expected {self.m} weights, got {t.numel()}")
        return t.contiguous()

    # ------------------------------------------------------------ customization
    def customize(self, w, storage: str = "int32", out: Metric | None = None, sync: bool = True,
                  method: str = "supernodal") -> Metric:
        """method "supernodal" (default) or "plain" (one launch per level,
        int32 only: the plain per-metric form kept for comparison)."""
        torch = self._torch
        lib = _lib.lib()
        wt = self.weights(w)
        dt = {"int32": torch.int32, "int64": torch.int64}[storage]
        if out is not None and out.up.dtype == dt:
            up, dn = out.up, out.dn
        else:
            up = torch.empty(self.m_plus, dtype=dt, device="cuda")
            dn = torch.empty(self.m_plus, dtype=dt, device="cuda")
        if method == "plain":
            if storage != "int32":
                raise ValueError("the plain customization stores int32")
            fn = lib.nwcch_customize_plain if sync else lib.nwcch_customize_plain_async
        else:
            fn = {("int32", True): lib.nwcch_customize, ("int32", False): lib.nwcch_customize_async,
                  ("int64", True): lib.nwcch_customize_i64,
                  ("int64", False): lib.nwcch_customize_i64_async}[storage, sync]
        sat = _status(fn(self.handle, wt.data_ptr(), up.data_ptr(), dn.data_ptr(), _stream(torch)), "customize")
        m = Metric(self, wt, up, dn, saturated=sat)
        if sat:
            warnings.warn(f"customization ({storage}) saturated: some values left the storage range",
                          SaturationWarning, stacklevel=2)
        return m

    def customize_batch(self, w, out: "MetricBatch | None" = None, sync: bool = True) -> "MetricBatch":
        """Customizes K metrics of this topology at once (int32 storage).

        w: K x m original weights (host array or device tensor). The result
        keeps the K metrics metric-major in two K x m+ tensors; every row is
        the metric nwcch_customize would produce for that row of w."""
        torch = self._torch
        if isinstance(w, torch.Tensor):
            wt = w.to(device="cuda", dtype=torch.int32).contiguous()
        else:
            rows = [self.weights(r) for r in np.asarray(w).reshape(-1, self.m)]
            wt = torch.stack(rows) if rows else torch.empty(0, self.m, dtype=torch.int32, device="cuda")
        wt = wt.reshape(-1, self.m)
        k = wt.shape[0]
        if k < 1:
            raise ValueError("need at least one metric")
        if out is not None and tuple(out.up.shape) == (k, self.m_plus):
            up, dn = out.up, out.dn
        else:
            up = torch.empty(k, self.m_plus, dtype=torch.int32, device="cuda")
            dn = torch.empty(k, self.m_plus, dtype=torch.int32, device="cuda")
        lib = _lib.lib()
        fn = lib.nwcch_customize_batch if sync else lib.nwcch_customize_batch_async
        sat = _status(fn(self.handle, k, wt.data_ptr(), up.data_ptr(), dn.data_ptr(), _stream(torch)),
                      "customize_batch")
        if sat:
            warnings.warn("batched customization saturated: some values left the int32 range",
                          SaturationWarning, stacklevel=2)
        return MetricBatch(self, wt, up, dn, saturated=sat)

    def negative_cycle_arcs_batch(self, b: "MetricBatch", out=None):
        """Per-metric negative-cycle arc counts of a batch (int64 CUDA tensor
        of K entries, enqueued on the current stream)."""
        torch = self._torch
        k = b.up.shape[0]
        if out is None:
            out = torch.empty(k, dtype=torch.int64, device="cuda")
        _lib.check(_lib.lib().nwcch_negative_cycle_arcs_batch_async(self.handle, k, b.up.data_ptr(), b.dn.data_ptr(),
                                                                    out.data_ptr(), _stream(torch)),
                   "negative_cycle_arcs_batch")
        return out

    def check(self) -> bool:
        """Status of asynchronous calls since the last check (True = saturated)."""
        return _status(_lib.lib().nwcch_check(self.handle, _stream(self._torch)), "check")

    def negative_cycle_arcs(self, m: Metric) -> int:
        lib = _lib.lib()
        fn = lib.nwcch_negative_cycle_arcs if m.storage == "int32" else lib.nwcch_negative_cycle_arcs_i64
        c = C.c_int64()
        _lib.check(fn(self.handle, m.up.data_ptr(), m.dn.data_ptr(), C.byref(c), _stream(self._torch)),
                   "negative_cycle_arcs")
        return int(c.value)

    def negative_cycle_arcs_async(self, m: Metric, out):
        """Enqueue the scan; the count lands in `out` (int64 CUDA tensor)."""
        if m.storage != "int32":
            raise ValueError("the enqueue-only scan reads int32 storage")
        _lib.check(_lib.lib().nwcch_negative_cycle_arcs_async(self.handle, m.up.data_ptr(), m.dn.data_ptr(),
                                                              out.data_ptr(), _stream(self._torch)),
                   "negative_cycle_arcs_async")

    def negative_loops(self, m: Metric) -> int:
        c = C.c_int64()
        _lib.check(_lib.lib().nwcch_negative_loops(self.handle, m.w.data_ptr(), C.byref(c), _stream(self._torch)),
                   "negative_loops")
        return int(c.value)

    # ------------------------------------------------------------ update
    def update(self, m: Metric, edge_idx, new_w):
        """Partial re-customization in place (python/cch.py:349-402).
        Returns the number of arcs re-evaluated."""
        torch = self._torch
        lib = _lib.lib()
        idx = np.ascontiguousarray(edge_idx, np.int64)
        val = np.asarray(new_w)
        if val.dtype.kind == "f" and not np.array_equal(val, np.rint(val)):
            raise ValueError("weights must be integral")
        val = np.ascontiguousarray(val, np.int64)
        if val.size and (val.max() >= _lib.INF32 or val.min() < -_lib.INF32):
            raise ValueError("weights must fit int32")
        val = val.astype(np.int32)
        stats = np.zeros(3, np.int64)
        changed = torch.empty(max(self.m_plus, 1), dtype=torch.int32, device="cuda")
        fn = lib.nwcch_update if m.storage == "int32" else lib.nwcch_update_i64
        sat = _status(fn(self.handle, m.w.data_ptr(), m.up.data_ptr(), m.dn.data_ptr(), _lib.ptr(idx), _lib.ptr(val),
                         idx.size, _lib.ptr(stats), changed.data_ptr(), _stream(torch)), "update")
        m.saturated = m.saturated or sat
        m.last_changed = changed[:int(stats[1])]
        m.stats = dict(evaluated=int(stats[0]), changed=int(stats[1]), changed_negative=int(stats[2]),
                       saturated=sat)
        return int(stats[0])

    # ------------------------------------------------------------ queries
    def query_batch(self, m: Metric, s_rank, t_rank, method: str = "supernodal", out=None, sync: bool = True):
        """int64 device tensor of distances (INT64_MAX = unreachable).
        method "supernodal" (batched kernel, shared-memory labels) or "plain"
        (one ancestor at a time, int32 storage only). sync=False only
        enqueues (supernodal, int32)."""
        torch = self._torch
        lib = _lib.lib()
        s = torch.as_tensor(np.asarray(s_rank) if not isinstance(s_rank, torch.Tensor) else s_rank)
        t = torch.as_tensor(np.asarray(t_rank) if not isinstance(t_rank, torch.Tensor) else t_rank)
        s = s.to(device="cuda", dtype=torch.int32).contiguous()
        t = t.to(device="cuda", dtype=torch.int32).contiguous()
        if s.numel() != t.numel():
            raise ValueError("s and t differ in length")
        if out is None:
            out = torch.empty(s.numel(), dtype=torch.int64, device="cuda")
        if method == "plain":
            if m.storage != "int32":
                raise ValueError("the plain query reads int32 storage")
            fn = lib.nwcch_query_batch_plain
        elif not sync:
            if m.storage != "int32":
                raise ValueError("the enqueue-only query reads int32 storage")
            fn = lib.nwcch_query_batch_async
        else:
            fn = lib.nwcch_query_batch if m.storage == "int32" else lib.nwcch_query_batch_i64
        _status(fn(self.handle, m.up.data_ptr(), m.dn.data_ptr(), s.data_ptr(), t.data_ptr(), s.numel(),
                   out.data_ptr(), _stream(torch)), "query_batch")
        return out

    def query_graph(self, m: Metric, size: int) -> "QueryGraph":
        """A captured CUDA graph of one batch of `size` queries on metric m
        (int32 storage): its launches are recorded once and replayed for
        every batch copied into its input buffers."""
        return QueryGraph(self, m, size)

    def query_paths(self, m: Metric, s_rank, t_rank, cap: int = 0):
        """Distances (int64 tensor) and shortest paths (python/cch.py:406-507)
        as (dist, off, path): path[off[i]:off[i+1]] are the ranks of pair i's
        path, s first (empty when unreachable). Synchronous."""
        torch = self._torch
        lib = _lib.lib()
        s = torch.as_tensor(np.asarray(s_rank) if not isinstance(s_rank, torch.Tensor) else s_rank)
        t = torch.as_tensor(np.asarray(t_rank) if not isinstance(t_rank, torch.Tensor) else t_rank)
        s = s.to(device="cuda", dtype=torch.int32).contiguous()
        t = t.to(device="cuda", dtype=torch.int32).contiguous()
        nq = s.numel()
        dist = torch.empty(nq, dtype=torch.int64, device="cuda")
        off = torch.empty(nq + 1, dtype=torch.int64, device="cuda")
        fn = lib.nwcch_query_paths if m.storage == "int32" else lib.nwcch_query_paths_i64
        need = C.c_int64()
        cap = max(int(cap), 64 * max(nq, 1))
        while True:
            path = torch.empty(cap, dtype=torch.int32, device="cuda")
            rc = fn(self.handle, m.up.data_ptr(), m.dn.data_ptr(), s.data_ptr(), t.data_ptr(), nq, dist.data_ptr(),
                    off.data_ptr(), path.data_ptr(), cap, C.byref(need), _stream(torch))
            if rc == -7 and need.value > cap:  # NWCCH_ERR_CAPACITY: retry with the exact size
                cap = int(need.value)
                continue
            _status(rc, "query_paths")
            return dist, off, path[:int(need.value)]

    # ------------------------------------------------------------ potential
    def potential(self, m: Metric, out=None):
        """CCH potential p(v) = min(0, min_u dist(u, v)) (cpp/cch.cpp:631-655),
        int64 CUDA tensor in RANK space."""
        torch = self._torch
        if out is None:
            out = torch.empty(max(self.n, 1), dtype=torch.int64, device="cuda")
        lib = _lib.lib()
        fn = lib.nwcch_potential if m.storage == "int32" else lib.nwcch_potential_i64
        if _status(fn(self.handle, m.up.data_ptr(), m.dn.data_ptr(), out.data_ptr(), _stream(torch)), "potential"):
            warnings.warn("potential saturated: some sums left the int64 range", SaturationWarning, stacklevel=2)
        return out[:self.n]


class QueryGraph:
    """Batches of a fixed size as one CUDA graph replay: the batched query's
    launches (range check, 32-bit and wide kernels) captured on a side stream
    over fixed input and output buffers. run() copies a batch in (device
    copies on the current stream), replays, and returns the output buffer
    (int64 distances, INT64_MAX = unreachable); the answers are those of
    query_batch on the same pairs."""

    def __init__(self, topo: DeviceTopology, m: Metric, size: int):
        torch = topo._torch
        if m.storage != "int32":
            raise ValueError("the captured query reads int32 storage")
        if size < 1:
            raise ValueError("size must be positive")
        self.topo, self.metric, self.size = topo, m, int(size)
        self.s = torch.zeros(self.size, dtype=torch.int32, device="cuda")
        self.t = torch.zeros(self.size, dtype=torch.int32, device="cuda")
        self.out = torch.empty(self.size, dtype=torch.int64, device="cuda")
        # warm-up outside the capture: plans, kernel attributes, scratch pools
        topo.query_batch(m, self.s, self.t, out=self.out, sync=False)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        with torch.cuda.stream(side):
            with torch.cuda.graph(self.graph, stream=side):
                topo.query_batch(m, self.s, self.t, out=self.out, sync=False)
        torch.cuda.synchronize()

    def run(self, s_rank, t_rank):
        torch = self.topo._torch
        s = torch.as_tensor(s_rank).to(device="cuda", dtype=torch.int32)
        t = torch.as_tensor(t_rank).to(device="cuda", dtype=torch.int32)
        if s.numel() != self.size or t.numel() != self.size:
            raise ValueError(f"batches of this graph hold {self.size} queries")
        self.s.copy_(s)
        self.t.copy_(t)
        self.graph.replay()
        return self.out


def distances_to_float(d) -> np.ndarray:
    """int64 distances (INT64_MAX = unreachable) -> float64 with inf."""
    a = d.cpu().numpy() if hasattr(d, "cpu") else np.asarray(d)
    f = a.astype(np.float64)
    f[a == _lib.INF64] = np.inf
    return f

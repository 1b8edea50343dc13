"""ctypes front end of the CPU oracle (oracle.c) - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this module. Values are int64 with ORC_INF = 2**63-1 for "no path".
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
INF = np.iinfo(np.int64).max

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> Path:
    """Compiles liboracle.so with the Makefile in this directory."""
    src = [HERE / "oracle.c", HERE / "oracle_battery.c", HERE / "oracle.h"]
    if force or not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime for p in src):
        subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(str(LIB))
            P, I64 = C.c_void_p, C.c_int64
            L.orc_customize.argtypes = [I64, P, P, I64, P, P, P, P, P]
            L.orc_customize.restype = None
            L.orc_customize_parallel.argtypes = [I64, P, P, I64, P, P, P, P, P, C.c_int]
            L.orc_customize_parallel.restype = I64
            L.orc_negative_cycle_arcs.argtypes = [I64, P, P]
            L.orc_negative_cycle_arcs.restype = I64
            L.orc_query.argtypes = [I64, I64, P, P, P, P, P, P, P, P, I64]
            L.orc_query.restype = I64
            L.orc_query_batch.argtypes = [I64, P, P, P, P, P, I64, P, P, P, C.c_int]
            L.orc_query_batch.restype = None
            L.orc_update.argtypes = [I64, P, P, I64, P, P, P, P, P, I64, P, P, P, P]
            L.orc_update.restype = None
            L.orc_update_index.argtypes = [I64, P, P, I64, P, P]
            L.orc_update_index.restype = P
            L.orc_update_indexed.argtypes = [P, P, P, P, I64, P, P, P, P]
            L.orc_update_indexed.restype = None
            L.orc_update_index_free.argtypes = [P]
            L.orc_update_index_free.restype = None
            L.orc_bellman_ford.argtypes = [I64, P, P, P, I64, P]
            L.orc_bellman_ford.restype = C.c_int
            L.orc_has_negative_cycle.argtypes = [I64, P, P, P]
            L.orc_potential.argtypes = [I64, P, P, P, P, P]
            L.orc_potential.restype = None
            L.orc_virtual_source_potential.argtypes = [I64, P, P, P, P]
            L.orc_virtual_source_potential.restype = C.c_int
            L.orc_has_negative_cycle.restype = C.c_int
            L.orc_query_path.argtypes = [I64, P, P, P, P, P, P, P, P, I64, I64, P, P, I64]
            L.orc_query_path.restype = I64
            L.orc_battery_customize.argtypes = [I64, P, P, I64, P, P, P, C.c_double]
            L.orc_battery_customize.restype = P
            L.orc_battery_pieces.argtypes = [P]
            L.orc_battery_pieces.restype = I64
            L.orc_battery_export.argtypes = [P, P, P, P]
            L.orc_battery_export.restype = None
            L.orc_battery_free.argtypes = [P]
            L.orc_battery_free.restype = None
            L.orc_battery_query_batch.argtypes = [I64, P, P, P, P, P, P, I64, P, P, P, P, C.c_int]
            L.orc_battery_query_batch.restype = None
            L.orc_battery_label_correcting.argtypes = [I64, P, P, P, C.c_double, I64, C.c_double, P]
            L.orc_battery_label_correcting.restype = None
            _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Topo:
    """Arrays of one contracted graph, converted once for the C calls."""

    def __init__(self, n, first, head, parent, e_arc, e_up):
        self.n = int(n)
        self.first = _c(first, np.int64)
        self.head = _c(head, np.int32)
        self.parent = _c(parent, np.int64)
        self.e_arc = _c(e_arc, np.int64)
        self.e_up = _c(e_up, np.int8)
        self.m_plus = int(self.first[-1])
        self.m = int(self.e_arc.size)

    @classmethod
    def from_dict(cls, t):
        return cls(t["n"], t["first"], t["head"], t["parent"], t["e_arc"], t["e_up"])

    def lower_lists(self):
        """tail int32[m+], and the arcs grouped by head (ascending tail):
        doff int64[n+1], darc int32[m+] (built once)."""
        if not hasattr(self, "_lower"):
            tail = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.first))
            darc = np.argsort(self.head, kind="stable").astype(np.int32)
            doff = np.zeros(self.n + 1, np.int64)
            np.cumsum(np.bincount(self.head, minlength=self.n), out=doff[1:])
            self._lower = (tail, doff, darc)
        return self._lower


def customize(T: Topo, w):
    w = _c(w, np.int32)
    up = np.empty(T.m_plus, np.int64)
    dn = np.empty(T.m_plus, np.int64)
    lib().orc_customize(T.n, _p(T.first), _p(T.head), T.m, _p(T.e_arc), _p(T.e_up), _p(w), _p(up), _p(dn))
    return up, dn


def customize_parallel(T: Topo, w, threads: int = 0):
    w = _c(w, np.int32)
    up = np.empty(T.m_plus, np.int64)
    dn = np.empty(T.m_plus, np.int64)
    lib().orc_customize_parallel(T.n, _p(T.first), _p(T.head), T.m, _p(T.e_arc), _p(T.e_up), _p(w), _p(up),
                                 _p(dn), int(threads))
    return up, dn


def negative_cycle_arcs(up, dn) -> int:
    up, dn = _c(up, np.int64), _c(dn, np.int64)
    return int(lib().orc_negative_cycle_arcs(up.size, _p(up), _p(dn)))


def query_batch(T: Topo, up, dn, s_rank, t_rank, threads: int = 0):
    up, dn = _c(up, np.int64), _c(dn, np.int64)
    s_rank, t_rank = _c(s_rank, np.int64), _c(t_rank, np.int64)
    out = np.empty(s_rank.size, np.int64)
    lib().orc_query_batch(T.n, _p(T.first), _p(T.head), _p(T.parent), _p(up), _p(dn), s_rank.size, _p(s_rank),
                          _p(t_rank), _p(out), int(threads))
    return out


def update(T: Topo, w, up, dn, edge_idx, new_w):
    """In place on w (int32), up, dn (int64). Returns (evaluated, changed arcs,
    changed arcs with up+dn<0)."""
    assert w.dtype == np.int32 and up.dtype == np.int64 and dn.dtype == np.int64
    edge_idx, new_w = _c(edge_idx, np.int64), _c(new_w, np.int32)
    stats = np.zeros(3, np.int64)
    changed = np.empty(max(T.m_plus, 1), np.int64)
    lib().orc_update(T.n, _p(T.first), _p(T.head), T.m, _p(T.e_arc), _p(T.e_up), _p(w), _p(up), _p(dn),
                     edge_idx.size, _p(edge_idx), _p(new_w), _p(stats), _p(changed))
    return int(stats[0]), changed[:stats[1]].copy(), int(stats[2])


class UpdateIndex:
    """The reference's update index (python/cch.py:289-347), built once per
    topology, and updates on it (python/cch.py:349-402): `update` has the
    module-level update's arguments and results, without the index build in
    every call (the reference builds it lazily, once)."""

    def __init__(self, T: Topo):
        self.T = T  # the index points into T's arrays
        self._h = lib().orc_update_index(T.n, _p(T.first), _p(T.head), T.m, _p(T.e_arc), _p(T.e_up))
        self._changed = np.empty(max(T.m_plus, 1), np.int64)

    def update(self, w, up, dn, edge_idx, new_w):
        assert self._h, "index freed"
        assert w.dtype == np.int32 and up.dtype == np.int64 and dn.dtype == np.int64
        edge_idx, new_w = _c(edge_idx, np.int64), _c(new_w, np.int32)
        stats = np.zeros(3, np.int64)
        lib().orc_update_indexed(self._h, _p(w), _p(up), _p(dn), edge_idx.size, _p(edge_idx), _p(new_w),
                                 _p(stats), _p(self._changed))
        return int(stats[0]), self._changed[:stats[1]].copy(), int(stats[2])

    def close(self):
        if self._h:
            lib().orc_update_index_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bellman_ford(n, off, tgt, w, s):
    off, tgt, w = _c(off, np.int64), _c(tgt, np.int32), _c(w, np.int32)
    dist = np.empty(n, np.int64)
    neg = lib().orc_bellman_ford(n, _p(off), _p(tgt), _p(w), int(s), _p(dist))
    return dist, bool(neg)


def has_negative_cycle(n, off, tgt, w) -> bool:
    off, tgt, w = _c(off, np.int64), _c(tgt, np.int32), _c(w, np.int32)
    return bool(lib().orc_has_negative_cycle(n, _p(off), _p(tgt), _p(w)))


def potential(T: Topo, up, dn):
    """cpp/cch.cpp:631-655: the CCH potential, rank space (int64[n])."""
    up, dn = _c(up, np.int64), _c(dn, np.int64)
    p = np.empty(T.n, np.int64)
    lib().orc_potential(T.n, _p(T.first), _p(T.head), _p(up), _p(dn), _p(p))
    return p


def virtual_source_potential(n, off, tgt, w):
    """Bellman-Ford from a virtual source (0-arcs to every vertex), original
    ids; None if a negative cycle exists."""
    off, tgt, w = _c(off, np.int64), _c(tgt, np.int32), _c(w, np.int32)
    p = np.empty(n, np.int64)
    return None if lib().orc_virtual_source_potential(n, _p(off), _p(tgt), _p(w), _p(p)) else p


def query_path(T: Topo, up, dn, s_rank: int, t_rank: int):
    """python/cch.py:406-507 in rank space: (distance, int64 array of ranks)."""
    up, dn = _c(up, np.int64), _c(dn, np.int64)
    tail, doff, darc = T.lower_lists()
    cap = 1024
    while True:
        path = np.empty(cap, np.int64)
        d = C.c_int64()
        n = lib().orc_query_path(T.n, _p(T.first), _p(T.head), _p(T.parent), _p(tail), _p(doff), _p(darc),
                                 _p(up), _p(dn), int(s_rank), int(t_rank), C.byref(d), _p(path), cap)
        if n >= 0:
            return int(d.value), path[:n].copy()
        cap = -n


def battery_customize(T: Topo, w, M: float):
    """python/cch_nb_battery.py:48-183: battery profiles of the float64 arc
    energies w for capacity M, canonical layout (cnt int32[2m+], off
    int64[2m+ + 1], pieces float64[total, 3] as (in, cost, out)); direction
    d = 2*arc + (0 up, 1 down)."""
    w = _c(w, np.float64)
    L = lib()
    h = L.orc_battery_customize(T.n, _p(T.first), _p(T.head), T.m, _p(T.e_arc), _p(T.e_up), _p(w), float(M))
    if not h:
        raise MemoryError("battery oracle: allocation failed")
    try:
        total = int(L.orc_battery_pieces(h))
        cnt = np.empty(2 * T.m_plus, np.int32)
        off = np.empty(2 * T.m_plus + 1, np.int64)
        pieces = np.empty((total, 3), np.float64)
        L.orc_battery_export(h, _p(cnt), _p(off), _p(pieces))
    finally:
        L.orc_battery_free(h)
    return cnt, off, pieces


def battery_query_batch(T: Topo, profiles, s_rank, t_rank, b0, threads: int = 0):
    """python/cch_nb_battery.py:296-343 per pair: best charge at t (-inf if
    infeasible)."""
    cnt, off, pieces = profiles
    cnt, off, pieces = _c(cnt, np.int32), _c(off, np.int64), _c(pieces, np.float64)
    s_rank, t_rank = _c(s_rank, np.int64), _c(t_rank, np.int64)
    b0 = _c(np.broadcast_to(b0, s_rank.shape), np.float64)
    out = np.empty(s_rank.size, np.float64)
    lib().orc_battery_query_batch(T.n, _p(T.first), _p(T.head), _p(T.parent), _p(cnt), _p(off), _p(pieces),
                                  s_rank.size, _p(s_rank), _p(t_rank), _p(b0), _p(out), int(threads))
    return out


def battery_label_correcting(n, off, tgt, w, M: float, s: int, b0: float):
    """python/cch_nb_battery.py:316-351: max charge at every vertex from s
    (original ids), float64[n] with -inf where infeasible."""
    off, tgt, w = _c(off, np.int64), _c(tgt, np.int32), _c(w, np.float64)
    soc = np.empty(n, np.float64)
    lib().orc_battery_label_correcting(n, _p(off), _p(tgt), _p(w), float(M), int(s), float(b0), _p(soc))
    return soc


def to_float(a):
    """int64 oracle values -> the reference's float64 convention (inf)."""
    a = np.asarray(a)
    out = a.astype(np.float64)
    out[a == INF] = np.inf
    return out


def from_float(a):
    """Reference float64 values (integral or inf) -> int64 oracle values."""
    a = np.asarray(a, dtype=np.float64)
    out = np.where(np.isinf(a), 0, a)
    if not np.array_equal(out, np.rint(out)):
        raise ValueError("non-integral reference value")
    out = out.astype(np.int64)
    out[np.isposinf(a)] = INF
    return out


def cpu_count() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1

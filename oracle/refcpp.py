"""ctypes front end of the reference C++ (cpp/cch.cpp) compiled unmodified
through ref_harness.cpp into _ref/libcchref.so - TEST INFRASTRUCTURE ONLY.

Available only where the reference checkout exists (the library is built from
its sources by `make -C oracle ref`). Used to generate golden fixtures and to
pin the oracle; never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libcchref.so"
# the reference checkout: NWCCH_REFERENCE_DIR names it (no default location)
REF_DIR = Path(os.environ["NWCCH_REFERENCE_DIR"]) if os.environ.get("NWCCH_REFERENCE_DIR") else None

_lib = None


def available() -> bool:
    return LIB.exists() or (REF_DIR is not None and (REF_DIR / "cpp" / "cch.cpp").exists())


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            if REF_DIR is None:
                raise RuntimeError("set NWCCH_REFERENCE_DIR to the reference checkout to build _ref/libcchref.so")
            subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_DIR={REF_DIR}"], check=True)
        L = C.CDLL(str(LIB))
        P, I64 = C.c_void_p, C.c_int64
        L.ref_create.restype = P
        L.ref_create.argtypes = [I64, P, P, P, P]
        L.ref_destroy.argtypes = [P]
        L.ref_order.argtypes = [P, I64, P]
        L.ref_set_order.argtypes = [P, P]
        L.ref_symbolic.restype = I64
        L.ref_symbolic.argtypes = [P, C.POINTER(I64), C.POINTER(I64)]
        L.ref_topology.argtypes = [P, P, P, P, P, P]
        L.ref_customize.restype = C.c_double
        L.ref_customize.argtypes = [P, P, P, P]
        L.ref_customize_parallel.restype = C.c_double
        L.ref_customize_parallel.argtypes = [P, P, P, P, C.c_int]
        L.ref_levels.restype = I64
        L.ref_levels.argtypes = [P]
        L.ref_negative_cycle_arcs.restype = I64
        L.ref_negative_cycle_arcs.argtypes = [P, P, P]
        L.ref_query_batch.restype = C.c_double
        L.ref_query_batch.argtypes = [P, P, P, I64, P, P, P]
        L.ref_johnson_potential.argtypes = [P, P, P]
        L.ref_dijkstra_batch.argtypes = [P, P, P, I64, P, P, P]
        L.ref_cch_potential.argtypes = [P, P, P, P]
        L.ref_cch_potential.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


class RefCCH:
    """One reference Graph + CCH, driven through the harness."""

    def __init__(self, g: dict):
        L = lib()
        self.n = int(g["n"])
        self.off = np.ascontiguousarray(g["off"], np.int64)
        self.tgt = np.ascontiguousarray(g["tgt"], np.int32)
        self.x = np.ascontiguousarray(g["x"], np.float64)
        self.y = np.ascontiguousarray(g["y"], np.float64)
        self.h = L.ref_create(self.n, _p(self.off), _p(self.tgt), _p(self.x), _p(self.y))
        self.m_plus = None

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ref_destroy(self.h)
            self.h = None

    def order(self, leaf: int = 64) -> np.ndarray:
        r = np.empty(self.n, np.int32)
        lib().ref_order(self.h, leaf, _p(r))
        self._rank = r
        return r.astype(np.int64)

    def set_order(self, rank):
        self._rank = np.ascontiguousarray(rank, np.int32)
        lib().ref_set_order(self.h, _p(self._rank))

    def symbolic(self) -> dict:
        d, t = C.c_int64(), C.c_int64()
        mp = lib().ref_symbolic(self.h, C.byref(d), C.byref(t))
        self.m_plus = mp
        first = np.empty(self.n + 1, np.int64)
        head = np.empty(mp, np.int32)
        parent = np.empty(self.n, np.int32)
        e_arc = np.empty(self.tgt.size, np.int64)
        e_up = np.empty(self.tgt.size, np.int8)
        lib().ref_topology(self.h, _p(first), _p(head), _p(parent), _p(e_arc), _p(e_up))
        return dict(n=self.n, rank=self._rank.astype(np.int64), first=first, head=head,
                    parent=parent.astype(np.int64), e_arc=e_arc, e_up=e_up, depth=d.value, triangles=t.value)

    def customize(self, w):
        w = np.ascontiguousarray(w, np.float64)
        up, dn = np.empty(self.m_plus), np.empty(self.m_plus)
        secs = lib().ref_customize(self.h, _p(w), _p(up), _p(dn))
        return up, dn, secs

    def customize_parallel(self, w, threads: int):
        w = np.ascontiguousarray(w, np.float64)
        up, dn = np.empty(self.m_plus), np.empty(self.m_plus)
        secs = lib().ref_customize_parallel(self.h, _p(w), _p(up), _p(dn), int(threads))
        return up, dn, secs

    def negative_cycle_arcs(self, up, dn) -> int:
        return int(lib().ref_negative_cycle_arcs(self.h, _p(np.ascontiguousarray(up)), _p(np.ascontiguousarray(dn))))

    def queries(self, up, dn, s, t):
        """Original vertex ids (the C++ Query::run maps them through rank)."""
        s = np.ascontiguousarray(s, np.int64)
        t = np.ascontiguousarray(t, np.int64)
        out = np.empty(s.size)
        secs = lib().ref_query_batch(self.h, _p(np.ascontiguousarray(up)), _p(np.ascontiguousarray(dn)), s.size,
                                     _p(s), _p(t), _p(out))
        return out, secs

    def cch_potential(self, up, dn):
        """The reference's CCH potential, original vertex ids (float64)."""
        pot = np.empty(self.n)
        lib().ref_cch_potential(self.h, _p(np.ascontiguousarray(up)), _p(np.ascontiguousarray(dn)), _p(pot))
        return pot

    def johnson_dijkstra(self, w, s, t):
        w = np.ascontiguousarray(w, np.float64)
        pot = np.empty(self.n)
        lib().ref_johnson_potential(self.h, _p(w), _p(pot))
        s = np.ascontiguousarray(s, np.int64)
        t = np.ascontiguousarray(t, np.int64)
        out = np.empty(s.size)
        lib().ref_dijkstra_batch(self.h, _p(w), _p(pot), s.size, _p(s), _p(t), _p(out))
        return out

"""ctypes binding of libnwcch.so (the C ABI declared in include/nwcch.h).

The library is built in-tree by ``negative-weight-cch_gb300/build.py``. There
is no fallback: if the library cannot be loaded, every entry point raises.

The weight-independent host preprocessing (``nwcch_undirected_csr``,
``nwcch_nested_dissection``, ``nwcch_symbolic``, ``nwcch_edge_arcs``, the graph
generation helpers) is bound from ``libnwcch_host.so``, which holds the same
host objects without device code: preparing a topology never maps the CUDA
library.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "_build" / "libnwcch.so"
HOST_LIB_PATH = PKG / "_build" / "libnwcch_host.so"

OK = 0
ERRORS = {
    -1: "invalid argument",
    -2: "allocation failed",
    -3: "CUDA runtime error",
    -4: "invalid topology",
    -5: "customized value outside int32 storage range",
    -6: "bounded device wait timed out",
    -7: "buffer capacity exceeded",
}
INF32 = 0x7FFFFFFF
INF64 = 0x7FFFFFFFFFFFFFFF


class NwcchError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__(f"{where}: {ERRORS.get(code, 'error')} (status {code})")


_lock = threading.Lock()
_lib = None
_host = None

P = C.c_void_p
I64 = C.c_int64
I32 = C.c_int32
PP = C.POINTER(C.c_void_p)
PI64 = C.POINTER(C.c_int64)

# name -> argtypes (restype is int unless listed in _VOID)
_SIGNATURES = {
    "nwcch_host_free": [P],
    "nwcch_undirected_csr": [I64, P, P, P, PP, PI64],
    "nwcch_nested_dissection": [I64, P, P, P, P, I64, C.c_int, P],
    "nwcch_symbolic": [I64, P, P, P, P, P, PP, PI64],
    "nwcch_edge_arcs": [I64, P, P, P, P, P, P, P],
    "nwcch_triangle_edges": [I64, I64, P, PP, PP, PI64],
    "nwcch_emst_mask": [I64, I64, P, P, P, P],
}
_VOID = {"nwcch_host_free"}
# bound from the host library (and from the full library too, where present)
_HOST = frozenset(_SIGNATURES)


def register(name: str, argtypes, restype=C.c_int):
    """Adds a signature (used by the modules that bind device entry points)."""
    _SIGNATURES[name] = argtypes
    if restype is None:
        _VOID.add(name)
    if _lib is not None:
        _bind(_lib, name)


def _bind(lib, name):
    f = getattr(lib, name)
    f.argtypes = _SIGNATURES[name]
    f.restype = None if name in _VOID else C.c_int


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"{LIB_PATH} is missing: build it with negative-weight-cch_gb300/build.py")
            handle = C.CDLL(str(LIB_PATH))
            for name in _SIGNATURES:
                _bind(handle, name)
            _lib = handle
    return _lib


def host_lib():
    """The host-only library (no device code): the preprocessing entry points."""
    global _host
    if _host is not None:
        return _host
    with _lock:
        if _host is None:
            if not HOST_LIB_PATH.exists():
                raise RuntimeError(f"{HOST_LIB_PATH} is missing: build it with negative-weight-cch_gb300/build.py")
            handle = C.CDLL(str(HOST_LIB_PATH))
            for name in _HOST:
                _bind(handle, name)
            _host = handle
    return _host


def check(code: int, where: str):
    if code != OK:
        raise NwcchError(code, where)


def ptr(a: np.ndarray | None):
    """Host pointer of a C-contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


def take_buffer(p: C.c_void_p, count: int, dtype) -> np.ndarray:
    """Copies a library-allocated buffer into numpy and frees it."""
    dtype = np.dtype(dtype)
    try:
        if count == 0:
            return np.empty(0, dtype)
        buf = (C.c_char * (count * dtype.itemsize)).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype, count=count).copy()
    finally:
        host_lib().nwcch_host_free(p)

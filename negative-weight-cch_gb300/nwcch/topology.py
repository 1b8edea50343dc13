"""Weight-independent preprocessing on the host, with the reference's names and
array layouts (python/cch_nb.py:22-524): undirected_csr, nested_dissection,
symbolic, edge_arcs, count_triangles. The work is done in C++ inside
libnwcch_host.so (the host objects of libnwcch.so without device code);
these wrappers only convert arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["undirected_csr", "nested_dissection", "symbolic", "edge_arcs", "count_triangles",
           "elimination_depth", "build_topology", "save_cache", "load_cache"]


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def undirected_csr(n, off, tgt):
    """Returns (noff int64[n+1], nbrs int32[...], rev int64[...]); rev is the
    position of u in v's list, as in the reference (cch_nb.py:22-71)."""
    lib = _lib.host_lib()
    off, tgt = _i64(off), _i32(tgt)
    noff = np.empty(n + 1, np.int64)
    nbr_p, slots = C.c_void_p(), C.c_int64()
    _lib.check(lib.nwcch_undirected_csr(n, _lib.ptr(off), _lib.ptr(tgt), _lib.ptr(noff),
                                        C.byref(nbr_p), C.byref(slots)), "undirected_csr")
    nbrs = _lib.take_buffer(nbr_p, slots.value, np.int32)
    # reverse slots (only the reference-shaped API needs them)
    owner = np.repeat(np.arange(n, dtype=np.int64), np.diff(noff))
    key_fwd = owner * n + nbrs
    key_rev = nbrs.astype(np.int64) * n + owner
    rev = np.searchsorted(key_fwd, key_rev).astype(np.int64)
    return noff, nbrs, rev


def nested_dissection(n, noff, nbrs, rev, x, y, leaf=64, threads=0):
    """rank[v] (int64, 0 = eliminated first); `rev` is accepted for signature
    compatibility with cch_nb.nested_dissection and not needed."""
    lib = _lib.host_lib()
    noff, nbrs = _i64(noff), _i32(nbrs)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    rank = np.empty(n, np.int32)
    _lib.check(lib.nwcch_nested_dissection(n, _lib.ptr(noff), _lib.ptr(nbrs), _lib.ptr(x), _lib.ptr(y),
                                           int(leaf), int(threads), _lib.ptr(rank)), "nested_dissection")
    return rank.astype(np.int64)


def symbolic(n, noff, nbrs, rank):
    """(first int64[n+1], head int32[m+] sorted per row, parent int64[n])."""
    lib = _lib.host_lib()
    noff, nbrs, rank32 = _i64(noff), _i32(nbrs), _i32(rank)
    first = np.empty(n + 1, np.int64)
    parent = np.empty(n, np.int32)
    head_p, mp = C.c_void_p(), C.c_int64()
    _lib.check(lib.nwcch_symbolic(n, _lib.ptr(noff), _lib.ptr(nbrs), _lib.ptr(rank32), _lib.ptr(first),
                                  _lib.ptr(parent), C.byref(head_p), C.byref(mp)), "symbolic")
    head = _lib.take_buffer(head_p, mp.value, np.int32)
    return first, head, parent.astype(np.int64)


def edge_arcs(n, off, tgt, rank, first, head):
    """(e_arc int64[m] with -1 for self-loops, e_up int8[m])."""
    lib = _lib.host_lib()
    off, tgt, rank32, first, head = _i64(off), _i32(tgt), _i32(rank), _i64(first), _i32(head)
    m = int(off[n])
    e_arc = np.empty(m, np.int64)
    e_up = np.empty(m, np.int8)
    _lib.check(lib.nwcch_edge_arcs(n, _lib.ptr(off), _lib.ptr(tgt), _lib.ptr(rank32), _lib.ptr(first),
                                   _lib.ptr(head), _lib.ptr(e_arc), _lib.ptr(e_up)), "edge_arcs")
    return e_arc, e_up


_lib.register("nwcch_edge_arcs_device", [C.c_int64] + [C.c_void_p] * 8)


def edge_arcs_device(n, off, tgt, rank, first, head):
    """The same mapping on the device (python/cch_nb.py:496-514): inputs are
    host arrays or CUDA tensors; returns CUDA tensors (e_arc int64, e_up int8)."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("edge_arcs_device needs a CUDA device")

    def dev(a, dt):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(device="cuda", dtype=dt).contiguous()
    off_d, tgt_d, rank_d = dev(off, torch.int64), dev(tgt, torch.int32), dev(rank, torch.int32)
    first_d, head_d = dev(first, torch.int64), dev(head, torch.int32)
    m = int(off_d[-1].item()) if n > 0 else 0
    e_arc = torch.empty(max(m, 1), dtype=torch.int64, device="cuda")
    e_up = torch.empty(max(m, 1), dtype=torch.int8, device="cuda")
    _lib.check(_lib.lib().nwcch_edge_arcs_device(int(n), off_d.data_ptr(), tgt_d.data_ptr(), rank_d.data_ptr(),
                                                  first_d.data_ptr(), head_d.data_ptr(), e_arc.data_ptr(),
                                                  e_up.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "edge_arcs_device")
    return e_arc[:m], e_up[:m]


def count_triangles(n, first, head):
    d = np.diff(np.asarray(first, dtype=np.int64))
    return int((d * (d - 1) // 2).sum())


def elimination_depth(parent):
    """Depth of every vertex in the elimination tree (root depth 0), by rank."""
    parent = np.asarray(parent, dtype=np.int64)
    n = parent.size
    depth = np.zeros(n, np.int64)
    for v in range(n - 1, -1, -1):  # parents have higher ranks
        p = parent[v]
        if p >= 0:
            depth[v] = depth[p] + 1
    return depth


def build_topology(g: dict, leaf: int = 64, rank=None, threads: int = 0) -> dict:
    """Full host pipeline for a graph dict from nwcch.graphs: order (unless
    `rank` is given), symbolic contraction and arc mapping."""
    n, off, tgt = g["n"], g["off"], g["tgt"]
    noff, nbrs, rev = undirected_csr(n, off, tgt)
    if rank is None:
        rank = nested_dissection(n, noff, nbrs, rev, g["x"], g["y"], leaf, threads)
    first, head, parent = symbolic(n, noff, nbrs, rank)
    e_arc, e_up = edge_arcs(n, off, tgt, rank, first, head)
    return dict(n=n, rank=np.asarray(rank, np.int64), first=first, head=head, parent=parent,
                e_arc=e_arc, e_up=e_up)


# ------------------------------------------------------------ topology cache

_GRAPH_KEYS = ("off", "tgt", "w", "L", "h", "x", "y")
_TOPO_KEYS = ("rank", "first", "head", "parent", "e_arc", "e_up")


def save_cache(path, key: str, g: dict, top: dict) -> bool:
    """Writes a graph and its topology as uncompressed .npy files under `path`
    (the role of the reference's rank_<name>.npy cache, python/run_nb.py:83-93,
    extended to the contracted topology). `key` names what was built (graph
    generator, size, seed, code version); a later load_cache with another key
    misses. Returns False, leaving no partial cache, when the write fails
    (a full disk is not an error of the caller)."""
    import json
    import shutil
    from pathlib import Path
    path = Path(path)
    tmp = path.with_name(path.name + ".tmp")
    try:
        shutil.rmtree(tmp, ignore_errors=True)
        tmp.mkdir(parents=True)
        for k in _GRAPH_KEYS:
            np.save(tmp / f"g_{k}.npy", np.asarray(g[k]))
        for k in _TOPO_KEYS:
            np.save(tmp / f"t_{k}.npy", np.asarray(top[k]))
        meta = {"key": key, "n": int(g["n"]), "kind": g.get("kind"), "seed": g.get("seed")}
        (tmp / "meta.json").write_text(json.dumps(meta))
        shutil.rmtree(path, ignore_errors=True)
        tmp.rename(path)
        return True
    except OSError:
        shutil.rmtree(tmp, ignore_errors=True)
        return False


def load_cache(path, key: str):
    """(g, top) from save_cache, or None when absent, unreadable or built under
    another key."""
    import json
    from pathlib import Path
    path = Path(path)
    try:
        meta = json.loads((path / "meta.json").read_text())
        if meta.get("key") != key:
            return None
        g = {k: np.load(path / f"g_{k}.npy") for k in _GRAPH_KEYS}
        g.update(n=int(meta["n"]), kind=meta.get("kind"), seed=meta.get("seed"))
        top = {k: np.load(path / f"t_{k}.npy") for k in _TOPO_KEYS}
        top["n"] = int(meta["n"])
        return g, top
    except (OSError, ValueError, KeyError):
        return None

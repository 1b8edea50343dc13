"""Drop-in replacement for the metric-dependent entry points of the
reference's python/cch_nb.py, with the same names and positional arguments:

    upw, dnw = customize(n, first, head, e_arc, e_up, w)      # cch_nb.py:529
    neg      = negative_cycle_arcs(upw, dnw)                  # cch_nb.py:566
    d        = query(s_rank, t_rank, first, head, parent,
                     upw, dnw, df, dr, mark, q)               # cch_nb.py:577

plus the weight-independent host functions (undirected_csr,
nested_dissection, symbolic, edge_arcs, count_triangles) re-exported from
nwcch.topology, and a batched query_batch.

Differences a caller sees:
* upw/dnw are CUDA tensors (int32, or int64 when int32 would saturate) that
  stay on the device; to_reference(upw, dnw) gives the reference's float64
  arrays with inf.
* Weights must be integral (int32 range); float arrays with integral values
  are accepted.
* query ignores the caller scratch df/dr/mark/q (kept for signature
  compatibility): labels live on the device.
* The topology arrays are uploaded on first use and cached by identity.
"""
from __future__ import annotations

import warnings
import weakref
from collections import OrderedDict

import numpy as np

from .device import DeviceTopology, Metric, SaturationWarning, distances_to_float
from .topology import count_triangles, edge_arcs, nested_dissection, symbolic, undirected_csr

__all__ = ["customize", "negative_cycle_arcs", "query", "query_batch", "to_reference", "undirected_csr",
           "nested_dissection", "symbolic", "edge_arcs", "count_triangles", "topology_for"]

_TOPO_CACHE: "OrderedDict[tuple, tuple]" = OrderedDict()
_TOPO_CACHE_SIZE = 4
_METRICS: "dict[int, weakref.ref]" = {}


def topology_for(n, first, head, e_arc, e_up, parent=None) -> DeviceTopology:
    """Device topology for these arrays (cached by the arrays' identity)."""
    key = (int(n), id(first), id(head), id(e_arc), id(e_up))
    hit = _TOPO_CACHE.get(key)
    if hit is not None:
        _TOPO_CACHE.move_to_end(key)
        return hit[0]
    topo = DeviceTopology(n, first, head, parent, e_arc, e_up)
    # keep the arrays alive so that their ids stay unique while cached
    _TOPO_CACHE[key] = (topo, (first, head, e_arc, e_up))
    while len(_TOPO_CACHE) > _TOPO_CACHE_SIZE:
        _TOPO_CACHE.popitem(last=False)[1][0].close()
    return topo


def _register(m: Metric):
    """Remembers which topology and weights produced upw while upw lives."""
    key = m.up.data_ptr()
    _METRICS[key] = (weakref.ref(m.up), weakref.ref(m.dn), m.topo, m.w, m.saturated)
    weakref.finalize(m.up, _METRICS.pop, key, None)
    return m


def _metric_of(upw) -> Metric:
    entry = _METRICS.get(upw.data_ptr()) if hasattr(upw, "data_ptr") else None
    if entry is None or entry[0]() is not upw or entry[1]() is None:
        raise ValueError("upw was not produced by nwcch.cch_nb.customize")
    return Metric(entry[2], entry[3], upw, entry[1](), saturated=entry[4])


class _Arcs(tuple):
    """(upw, dnw) that also keeps its Metric alive."""
    metric: Metric


def customize(n, first, head, e_arc, e_up, w, storage: str = "auto"):
    """Customized (upw, dnw) of metric w over the contracted graph
    (python/cch_nb.py:529-563). storage: "int32", "int64", or "auto"
    (int32, redone in int64 if int32 saturates)."""
    topo = topology_for(n, first, head, e_arc, e_up)
    if storage == "auto":
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", SaturationWarning)
            m = topo.customize(w, "int32")
        if m.saturated:
            m = topo.customize(w, "int64")
    else:
        m = topo.customize(w, storage)
    _register(m)
    out = _Arcs((m.up, m.dn))
    out.metric = m
    return out


def negative_cycle_arcs(upw, dnw) -> int:
    """Arcs with upw + dnw < 0 (python/cch_nb.py:566-572)."""
    m = _metric_of(upw)
    if m.dn is not dnw:
        raise ValueError("upw and dnw come from different customizations")
    return m.topo.negative_cycle_arcs(m)


def query(s_rank, t_rank, first, head, parent, upw, dnw, df=None, dr=None, mark=None, q=None) -> float:
    """Distance from rank s_rank to rank t_rank (python/cch_nb.py:577-615);
    inf if t is unreachable."""
    m = _metric_of(upw)
    d = m.topo.query_batch(m, np.array([int(s_rank)]), np.array([int(t_rank)]))
    return float(distances_to_float(d)[0])


def query_batch(s_ranks, t_ranks, upw, dnw) -> np.ndarray:
    """Distances (float64, inf = unreachable) for rank pairs, one launch."""
    m = _metric_of(upw)
    return distances_to_float(m.topo.query_batch(m, s_ranks, t_ranks))


def to_reference(upw, dnw):
    """The reference's arrays: float64 with inf."""
    return _metric_of(upw).to_reference()

"""GPU counterpart of the reference's CCH class (python/cch.py) for the
metric-dependent operations: customize, update_edges, has_negative_cycle,
update_created_negative_cycle, query.

The weight-independent phase (order, chordal completion, arc mapping) runs on
the host in C++ (nwcch.topology); everything metric-dependent runs in
libnwcch's kernels on the resident topology. Weights are integers.
"""
from __future__ import annotations

import numpy as np

from . import topology as T
from .device import DeviceTopology, Metric, distances_to_float

__all__ = ["CCH"]


class CCH:
    """n, off (int64[n+1]), tgt (int32[m]): the directed graph in CSR form
    (edge index = CSR position, as the reference's g.adj order). Either an
    explicit `order` (rank per vertex) or coordinates x, y for the
    nested-dissection order."""

    def __init__(self, n, off, tgt, x=None, y=None, leaf=64, order=None, storage="int64", threads=0):
        g = dict(n=int(n), off=np.asarray(off, np.int64), tgt=np.asarray(tgt, np.int32), x=x, y=y)
        if order is None and (x is None or y is None):
            raise ValueError("need coordinates or an explicit order")
        top = T.build_topology(g, leaf=leaf, rank=order, threads=threads)
        self.n = int(n)
        self.off, self.tgt = g["off"], g["tgt"]
        self.rank = top["rank"]
        self.first, self.head, self.parent = top["first"], top["head"], top["parent"]
        self.edge_arc, self.edge_dir = top["e_arc"], top["e_up"]
        self.m = int(self.first[-1])
        self.loop_edges = np.nonzero(self.edge_arc < 0)[0]
        self.storage = storage
        self.dev = DeviceTopology(self.n, self.first, self.head, self.parent, self.edge_arc, self.edge_dir)
        self.depth = int(self.dev.depth)
        self.triangles = int(self.dev.triangles)
        self.metric: Metric | None = None
        self.last_changed = np.empty(0, np.int64)

    @classmethod
    def from_graph(cls, g: dict, **kw) -> "CCH":
        return cls(g["n"], g["off"], g["tgt"], x=g.get("x"), y=g.get("y"), **kw)

    # ------------------------------------------------------------ customization
    def customize(self, w) -> list:
        """Full customization (python/cch.py:249-287). Returns the arcs that
        witness a negative cycle ([-1] for a negative self-loop), like the
        reference."""
        self.metric = self.dev.customize(w, self.storage)
        if self.dev.negative_loops(self.metric) > 0:
            return [-1]
        return self._negative_arcs()

    def _negative_arcs(self) -> list:
        if self.dev.negative_cycle_arcs(self.metric) == 0:
            return []
        up, dn = self.metric.to_numpy()
        inf = np.iinfo(np.int64).max
        fin = (up != inf) & (dn != inf)
        s = up[fin].astype(object) + dn[fin].astype(object)
        return [int(a) for a, v in zip(np.nonzero(fin)[0], s) if v < 0]

    @property
    def up(self):
        return self.metric.to_reference()[0]

    @property
    def down(self):
        return self.metric.to_reference()[1]

    # ------------------------------------------------------------ updates
    def update_edges(self, changes) -> int:
        """changes = [(edge_index, new_weight)] (python/cch.py:349-402).
        Returns the number of arcs re-evaluated."""
        if self.metric is None:
            raise RuntimeError("customize first")
        idx = np.array([int(k) for k, _ in changes], np.int64)
        val = np.array([w for _, w in changes])
        ev = self.dev.update(self.metric, idx, val)
        self.last_changed = self.metric.last_changed.cpu().numpy().astype(np.int64)
        return ev

    def has_negative_cycle(self) -> bool:
        """python/cch.py:662-664."""
        return self.dev.negative_loops(self.metric) > 0 or self.dev.negative_cycle_arcs(self.metric) > 0

    def update_created_negative_cycle(self) -> bool:
        """Checks only the arcs the last update changed (python/cch.py:666-671)."""
        return self.dev.negative_loops(self.metric) > 0 or self.metric.stats.get("changed_negative", 0) > 0

    def query_path(self, s, t):
        """python/cch.py:406-507: (distance, [original vertices of a shortest
        path]) with the reference's choice among equal-length paths; (inf, [])
        if t is unreachable."""
        dist, off, path = self.dev.query_paths(self.metric, self.rank[[s]], self.rank[[t]])
        inv = np.empty_like(self.rank)
        inv[self.rank] = np.arange(self.n)
        p = path.cpu().numpy()
        return float(distances_to_float(dist)[0]), [int(v) for v in inv[p]]

    def potential(self) -> np.ndarray:
        """python/cch.py:734-755: the feasible potential p(v) = min(0,
        min_u dist(u, v)) read off the customized metric, per ORIGINAL vertex
        (float64, as the reference)."""
        p = self.dev.potential(self.metric).cpu().numpy()
        return p[self.rank].astype(np.float64)

    # ------------------------------------------------------------ queries
    def query(self, s, t) -> float:
        """Distance between ORIGINAL vertex ids s and t (inf if unreachable)."""
        return float(self.query_batch([s], [t])[0])

    def query_batch(self, s, t) -> np.ndarray:
        s = np.asarray(s, np.int64)
        t = np.asarray(t, np.int64)
        d = self.dev.query_batch(self.metric, self.rank[s], self.rank[t])
        return distances_to_float(d)

"""GPU counterpart of the reference's BatteryCCH (python/cch_battery.py): the
battery-constrained layer over a CCH, customized and queried on the device.

    from nwcch.cch import CCH
    from nwcch.cch_battery import BatteryCCH
    c = CCH.from_graph(g)
    bc = BatteryCCH(c)
    largest, mean = bc.customize(w, M)        # python/cch_battery.py customize(g, M)
    soc = bc.query(s, t, b0)                   # best charge at t, -inf if infeasible

Differences a caller sees:
* customize takes the arc energies as the reference's Graph object, as an
  array in CSR edge order (the reference's g.adj order), or as a graph dict
  holding them under "w_energy";
* the profiles are those of the reference's Numba customization
  (python/cch_nb_battery.py: candidates merged for ascending lowest vertex);
  the pure-Python class merges in its triangle-list order, so near-equal
  pieces may differ while every answer agrees within the reference's
  tolerance;
* profiles stay on the device; profiles() copies them out as lists of
  (in, cost, out) per shortcut direction.
"""
from __future__ import annotations

import numpy as np

from . import battery as _bat

__all__ = ["BatteryCCH", "energies_of"]


def energies_of(g) -> np.ndarray:
    """float64 arc energies in edge order from an array, a graph dict
    ("w_energy") or the reference's Graph object (g.adj[u] = [(v, w), ...],
    edge index = position in that order, python/graphs.py:21-33)."""
    if hasattr(g, "adj"):
        return np.fromiter((w for nb in g.adj for _, w in nb), np.float64)
    if isinstance(g, dict):
        g = g["w_energy"]
    return np.ascontiguousarray(g, np.float64)


class BatteryCCH:
    """Battery profiles over an nwcch.cch.CCH (its resident topology)."""

    def __init__(self, cch):
        self.c = cch
        self.M = None
        self._prof = None

    def customize(self, w, M):
        """Profiles for energies w and capacity M; returns the reference's
        (largest profile, mean pieces per direction)."""
        w = energies_of(w)
        if self._prof is not None:
            self._prof.free()
        self._prof = _bat.customize(self.c.dev, w, float(M))
        self.M = float(M)
        nd = 2 * self.c.m
        return self._prof.largest, (self._prof.pieces / nd if nd else 0.0)

    def query(self, s, t, b0) -> float:
        """Best state of charge at t when leaving s with b0, -inf if t is not
        reachable with that charge (original vertex ids)."""
        if self._prof is None:
            raise RuntimeError("customize first")
        r = self._prof.query(np.array([self.c.rank[s]]), np.array([self.c.rank[t]]), float(b0))
        return float(r.cpu().numpy()[0])

    def query_batch(self, s, t, b0) -> np.ndarray:
        """query for arrays of original vertex ids (b0 scalar or per pair)."""
        if self._prof is None:
            raise RuntimeError("customize first")
        return self._prof.query(self.c.rank[np.asarray(s)], self.c.rank[np.asarray(t)], b0).cpu().numpy()

    def profiles(self):
        """(up, down): per shortcut arc, the list of (in, cost, out) pieces of
        each direction, as the reference's BatteryCCH.up / .down."""
        cnt, off, pieces = self._prof.export()
        up = [[tuple(p) for p in pieces[off[2 * a]:off[2 * a + 1]]] for a in range(self.c.m)]
        down = [[tuple(p) for p in pieces[off[2 * a + 1]:off[2 * a + 2]]] for a in range(self.c.m)]
        return up, down

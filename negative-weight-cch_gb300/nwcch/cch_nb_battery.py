"""Drop-in replacement for the reference's python/cch_nb_battery.py, same
names and positional arguments:

    prof = battery_customize(n, first, head, e_arc, e_up, w, M)   # :48
    cnt, I1, C1, O1, pst, PI, PC, PO = prof
    b    = battery_query(s_rank, t_rank, b0, first, head, parent,
                         cnt, I1, C1, O1, pst, PI, PC, PO,
                         soc, dsoc, mark, q)                       # :296
    h    = size_histogram(cnt)                                     # :354

plus battery_query_batch for many (s, t, b0) in one launch.

The customization and the queries run on the device (nwcch.battery); the
returned arrays are the reference's layout copied to the host - single
pieces inline in (I1, C1, O1), longer profiles at [pst, pst + cnt) of
(PI, PC, PO) - with the same pieces in the same order. battery_query finds
the device profiles through the `cnt` array it was given (it must come from
battery_customize) and ignores the caller scratch soc/dsoc/mark/q.
"""
from __future__ import annotations

import weakref

import numpy as np

from . import battery as _bat
from .cch_nb import topology_for

__all__ = ["battery_customize", "battery_query", "battery_query_batch", "size_histogram", "profiles_of"]

_PROFILES: "dict[int, tuple]" = {}


class _Profiles(tuple):
    """The reference's 8 arrays; .device holds the device profiles."""
    device: _bat.BatteryProfiles


def _reference_layout(cnt, off, pieces):
    nd = cnt.size
    single = cnt == 1
    I1, C1, O1 = np.zeros(nd), np.zeros(nd), np.zeros(nd)
    idx = off[:-1][single]
    I1[single], C1[single], O1[single] = pieces[idx, 0], pieces[idx, 1], pieces[idx, 2]
    multi = cnt > 1
    pst = np.full(nd, -1, np.int64)
    sizes = np.where(multi, cnt, 0).astype(np.int64)
    starts = np.zeros(nd, np.int64)
    np.cumsum(sizes[:-1], out=starts[1:])
    pst[multi] = starts[multi]
    sel = np.repeat(off[:-1][multi], cnt[multi]) + (np.arange(int(sizes.sum())) -
                                                    np.repeat(starts[multi], cnt[multi]))
    PI, PC, PO = pieces[sel, 0].copy(), pieces[sel, 1].copy(), pieces[sel, 2].copy()
    return cnt, I1, C1, O1, pst, PI, PC, PO


def battery_customize(n, first, head, e_arc, e_up, w, M):
    """python/cch_nb_battery.py:48-183 on the device; returns the reference's
    (cnt, I1, C1, O1, pst, PI, PC, PO)."""
    topo = topology_for(n, first, head, e_arc, e_up)
    dev = _bat.customize(topo, w, M)
    cnt, off, pieces = dev.export()
    out = _Profiles(_reference_layout(cnt, off, pieces))
    out.device = dev
    key = id(out[0])
    _PROFILES[key] = (weakref.ref(out[0]), dev)
    weakref.finalize(out[0], _PROFILES.pop, key, None)
    return out


def profiles_of(cnt) -> _bat.BatteryProfiles:
    """The device profiles whose counts array is `cnt`."""
    entry = _PROFILES.get(id(cnt))
    if entry is None or entry[0]() is not cnt:
        raise ValueError("cnt was not produced by nwcch.cch_nb_battery.battery_customize")
    return entry[1]


def battery_query(s_rank, t_rank, b0, first, head, parent, cnt, I1=None, C1=None, O1=None, pst=None, PI=None,
                  PC=None, PO=None, soc=None, dsoc=None, mark=None, q=None) -> float:
    """Best state of charge at t leaving s with b0, -inf if infeasible
    (python/cch_nb_battery.py:296-343)."""
    dev = profiles_of(cnt)
    return float(dev.query(np.array([int(s_rank)]), np.array([int(t_rank)]), float(b0)).cpu().numpy()[0])


def battery_query_batch(s_ranks, t_ranks, b0, cnt) -> np.ndarray:
    """battery_query for many pairs in one launch (float64, -inf infeasible)."""
    return profiles_of(cnt).query(s_ranks, t_ranks, b0).cpu().numpy()


def size_histogram(cnt) -> np.ndarray:
    """python/cch_nb_battery.py:354-371: directions with 0, 1, 2-5, 6-10,
    11-50, 51-100, >100 pieces, and the largest profile."""
    cnt = np.asarray(cnt)
    edges = [(0, 0), (1, 1), (2, 5), (6, 10), (11, 50), (51, 100), (101, 1 << 31)]
    h = np.array([np.count_nonzero((cnt >= lo) & (cnt <= hi)) for lo, hi in edges] + [0], np.int64)
    h[7] = int(cnt.max()) if cnt.size else 0
    return h

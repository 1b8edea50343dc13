"""Battery-constrained profiles on the device (libnwcch battery.cu).

A customization turns float64 arc energies and a battery capacity M into
per-direction profiles of (in, cost, out) pieces, the reference's profiles
piece for piece (python/cch_nb_battery.py:48-183); queries return the best
state of charge at t when leaving s with charge b0, -inf if infeasible
(python/cch_nb_battery.py:296-343). Everything runs on the device; there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .device import DeviceTopology, _stream, _torch

P, I64, I32 = C.c_void_p, C.c_int64, C.c_int32

_lib.register("nwcch_battery_customize", [P, P, C.c_double, P, C.POINTER(C.c_void_p)])
_lib.register("nwcch_battery_info", [P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)])
_lib.register("nwcch_battery_export", [P, P, P, P])
_lib.register("nwcch_battery_query", [P, P, P, P, P, I64, P, P])
_lib.register("nwcch_battery_free", [P], restype=None)


class BatteryProfiles:
    """Device-resident profiles of one (topology, energies, capacity)."""

    def __init__(self, topo: DeviceTopology, handle, M: float):
        self.topo = topo
        self._h = handle
        self.M = float(M)
        pieces, largest = C.c_int64(), C.c_int32()
        _lib.check(_lib.lib().nwcch_battery_info(self.handle, C.byref(pieces), C.byref(largest)), "battery_info")
        self.pieces = int(pieces.value)
        self.largest = int(largest.value)

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("battery profiles are freed")
        return self._h

    def free(self):
        if getattr(self, "_h", None) is not None:
            _lib.lib().nwcch_battery_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def export(self, pieces: bool = True):
        """Host copy in direction order: cnt int32[2m+], off int64[2m+ + 1],
        pieces float64[total, 3] as (in, cost, out) (None if not asked)."""
        nd = 2 * self.topo.m_plus
        cnt = np.empty(nd, np.int32)
        off = np.empty(nd + 1, np.int64)
        pc = np.empty((self.pieces, 3), np.float64) if pieces else None
        _lib.check(_lib.lib().nwcch_battery_export(self.handle, _lib.ptr(cnt), _lib.ptr(off), _lib.ptr(pc)),
                   "battery_export")
        return cnt, off, pc

    def size_histogram(self) -> np.ndarray:
        """python/cch_nb_battery.py:354-371: directions with 0, 1, 2-5, 6-10,
        11-50, 51-100, >100 pieces, and the largest profile."""
        cnt, _, _ = self.export(pieces=False)
        edges = [(0, 0), (1, 1), (2, 5), (6, 10), (11, 50), (51, 100), (101, 1 << 31)]
        h = np.array([np.count_nonzero((cnt >= lo) & (cnt <= hi)) for lo, hi in edges] + [0], np.int64)
        h[7] = int(cnt.max()) if cnt.size else 0
        return h

    def query(self, s_rank, t_rank, b0, out=None, sync: bool = True):
        """Best charge at t leaving s with b0 per pair (float64 CUDA tensor,
        -inf if infeasible). s/t are rank ids; b0 a scalar or one per pair."""
        torch = _torch()
        s = torch.as_tensor(np.asarray(s_rank) if not isinstance(s_rank, torch.Tensor) else s_rank)
        t = torch.as_tensor(np.asarray(t_rank) if not isinstance(t_rank, torch.Tensor) else t_rank)
        s = s.to(device="cuda", dtype=torch.int32).contiguous()
        t = t.to(device="cuda", dtype=torch.int32).contiguous()
        if s.numel() != t.numel():
            raise ValueError("s and t differ in length")
        if isinstance(b0, torch.Tensor):
            b = b0.to(device="cuda", dtype=torch.float64).reshape(-1)
        else:
            b = torch.as_tensor(np.broadcast_to(np.asarray(b0, np.float64), (s.numel(),)).copy()).cuda()
        if b.numel() not in (1, s.numel()):
            # the kernel reads one start charge per query
            raise ValueError(f"b0 has {b.numel()} values for {s.numel()} queries (expected 1 or {s.numel()})")
        b = b.expand(s.numel()).contiguous() if b.numel() == 1 else b.contiguous()
        if out is None:
            out = torch.empty(max(s.numel(), 1), dtype=torch.float64, device="cuda")
        _lib.check(_lib.lib().nwcch_battery_query(self.topo.handle, self.handle, s.data_ptr(), t.data_ptr(),
                                                   b.data_ptr(), s.numel(), out.data_ptr(), _stream(torch)),
                   "battery_query")
        if sync:
            torch.cuda.current_stream().synchronize()
        return out[:s.numel()]


def energies(topo: DeviceTopology, w):
    """float64 device tensor of the original arcs' energies."""
    torch = _torch()
    if isinstance(w, torch.Tensor):
        t = w.to(device="cuda", dtype=torch.float64)
    else:
        t = torch.from_numpy(np.ascontiguousarray(w, np.float64)).to("cuda")
    if t.numel() != topo.m:
        raise ValueError(f"expected {topo.m} energies, got {t.numel()}")
    return t.contiguous()


def customize(topo: DeviceTopology, w, M: float) -> BatteryProfiles:
    """Profiles of energies w (float64[m], original arc order) for battery
    capacity M (python/cch_nb_battery.py:48-183)."""
    torch = _torch()
    wt = energies(topo, w)
    h = C.c_void_p()
    _lib.check(_lib.lib().nwcch_battery_customize(topo.handle, wt.data_ptr(), float(M), _stream(torch),
                                                  C.byref(h)), "battery_customize")
    return BatteryProfiles(topo, h, M)

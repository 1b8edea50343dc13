"""nwcch - the metric-dependent hot path of Customizable Contraction
Hierarchies with negative arc weights, on GB300 (sm_103a).

Modules
  cch_nb    drop-in for the reference's python/cch_nb.py entry points
  cch       GPU counterpart of the reference's CCH class (updates, cycles)
  device    DeviceTopology / Metric over the C ABI (include/nwcch.h)
  topology  weight-independent host preprocessing (C++)
  graphs    seeded synthetic workloads
"""
from ._lib import NwcchError, lib  # noqa: F401

__all__ = ["NwcchError", "lib"]

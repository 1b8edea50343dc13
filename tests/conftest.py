"""Shared test set-up: import paths, the `gpu` marker, fixture loaders."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "negative-weight-cch_gb300"
for p in (PKG, ROOT / "oracle", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and runs the sm_103a kernels")


@pytest.fixture(scope="session")
def built_lib():
    import build as nwbuild  # negative-weight-cch_gb300/build.py
    nwbuild.build()
    from nwcch import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc  # oracle/oracle.py
    orc.lib()
    return orc


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def battery_cases():
    """battery.npz as a list of (graph dict, [per-capacity dicts])."""
    B = load_golden("battery.npz")
    out = []
    for i in range(int(B["cases"])):
        pre = f"c{i}_"
        g = {k[len(pre):]: v for k, v in B.items() if k.startswith(pre) and not k[len(pre):].startswith("m")}
        caps = []
        for mi in range(int(B["capacities"])):
            p2 = f"{pre}m{mi}_"
            caps.append({k[len(p2):]: v for k, v in B.items() if k.startswith(p2)})
        out.append((g, caps))
    return out


def family_case(F: dict, i: int) -> dict:
    pre = f"c{i}_"
    out = {k[len(pre):]: v for k, v in F.items() if k.startswith(pre)}
    steps = []
    for si in range(int(out["steps"])):
        sp = f"s{si}_"
        steps.append({k[len(sp):]: v for k, v in out.items() if k.startswith(sp)})
    out["step_list"] = steps
    return out


def i32_to_i64(a):
    """int32 storage with INT32_MAX = inf -> int64 with INT64_MAX = inf."""
    a = np.asarray(a)
    out = a.astype(np.int64)
    out[a == np.iinfo(np.int32).max] = np.iinfo(np.int64).max
    return out


@pytest.fixture(scope="session")
def gpu(built_lib):
    """torch with a CUDA device; a GPU test without one fails (no fallback)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return torch

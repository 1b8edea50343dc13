"""Builds libnwcch.so (CUDA kernels for sm_103a + host C++ + the C ABI) in-tree,
and libnwcch_host.so (the weight-independent host preprocessing alone).

    python negative-weight-cch_gb300/build.py [--force]

Every .cu is compiled by nvcc for sm_103a only, every .cpp by g++, in
parallel; the shared library links the CUDA runtime statically so that it
loads with no GPU present. The host library holds only the .cpp objects (no
device code, no CUDA runtime): ordering, symbolic contraction, arc mapping and
graph generation helpers, for processes that prepare topologies without
touching the GPU. The build is skipped when a stamp of the sources and flags
is unchanged.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libnwcch.so"
HOST_LIB = OUT_DIR / "libnwcch_host.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stamp() -> str:
    h = hashlib.sha256()
    for p in _sources() + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "nwcch.h"]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    stamp_file = OUT_DIR / "stamp"
    stamp = _stamp()
    if (not force and LIB.exists() and HOST_LIB.exists() and stamp_file.exists()
            and stamp_file.read_text() == stamp):
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]

    def compile_one(src: Path):
        obj = OUT_DIR / (src.name + ".o")
        if src.suffix == ".cu":
            cmd = [nvcc, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
        log = _run(cmd)
        if verbose and log.strip():
            print(log)
        return obj

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
          "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    host_objs = [o for o, src in zip(objs, _sources()) if src.suffix == ".cpp"]
    tmp = HOST_LIB.with_suffix(".so.tmp")
    _run([os.environ.get("CXX", "g++"), "-shared", "-pthread", "-o", str(tmp), *map(str, host_objs)])
    os.replace(tmp, HOST_LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)

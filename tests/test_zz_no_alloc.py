"""The allocation-free query entry point (nwcch_query_batch_noalloc).

Callers that cannot allocate device memory (a serving loop whose memory is
all handed to resident metrics, an application whose own allocator owns the
GPU) use this entry point; it keeps its scratch in a fixed array inside the
library. Here it is called through the C ABI and must return exactly what
nwcch_query_batch returns, on two calls in a row (the second one reuses the
scratch the first one left behind). The file sorts last so that a run which
stops at the first failure has run everything else first.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _bind(lib):
    P = C.c_void_p
    f = lib.nwcch_query_batch_noalloc
    f.argtypes = [P, P, P, P, P, C.c_int64, P, P]
    f.restype = C.c_int
    return f


def test_noalloc_queries_match_the_allocating_entry_point(gpu):
    torch = gpu
    from nwcch import _lib
    from nwcch import graphs as G
    from nwcch import topology as T
    from nwcch.device import DeviceTopology

    lib = _lib.lib()
    noalloc = _bind(lib)
    cases = []
    z = load_golden("grid64.npz")
    cases.append((DeviceTopology(int(z["n"]), z["first"], z["head"], z["parent"], z["e_arc"], z["e_up"]), z["w"],
                  z["rank"][z["qs"]], z["rank"][z["qt"]], z["ans"]))
    g = G.delaunay(30_000, seed=12)
    top = T.build_topology(g)
    s, t = G.random_pairs(g["n"], 5_000, seed=4)
    cases.append((DeviceTopology.from_dict(top), g["w"], top["rank"][s], top["rank"][t], None))
    # a tree deep enough (depth > 345) that the fixed scratch holds fewer
    # blocks of warps than the batch wants: warps then answer several queries
    # each, reusing one scratch slot
    g = G.delaunay(60_000, seed=12)
    top = T.build_topology(g)
    assert T.elimination_depth(top["parent"]).max() > 345
    s, t = G.random_pairs(g["n"], 6_000, seed=5)
    cases.append((DeviceTopology.from_dict(top), g["w"], top["rank"][s], top["rank"][t], None))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for topo, w, qs, qt, golden in cases:
        m = topo.customize(w, "int32")
        want = topo.query_batch(m, qs, qt).cpu().numpy()
        if golden is not None:
            assert np.array_equal(want, golden)
        s_dev = torch.from_numpy(np.ascontiguousarray(qs, np.int32)).cuda()
        t_dev = torch.from_numpy(np.ascontiguousarray(qt, np.int32)).cuda()
        for _ in range(2):
            out = torch.full((s_dev.numel(),), -7, dtype=torch.int64, device="cuda")
            rc = noalloc(topo.handle, m.up.data_ptr(), m.dn.data_ptr(), s_dev.data_ptr(), t_dev.data_ptr(),
                         s_dev.numel(), out.data_ptr(), stream)
            assert rc == 0, rc
            assert np.array_equal(out.cpu().numpy(), want)


def test_noalloc_rejects_a_tree_too_deep_for_the_fixed_scratch(gpu):
    """A path eliminated from one end has depth n - 1; at 420,000 vertices a
    block of 4 warps needs 4 * 8 * (2.5 * 420,000 + 1) bytes, more than the
    32 MiB array, so the call returns NWCCH_ERR_CAPACITY before launching."""
    torch = gpu
    from nwcch import _lib
    from nwcch.device import DeviceTopology

    n = 420_000
    per_warp_words = 2 * n + (n + 1) // 2 + 1
    assert 4 * per_warp_words > (4 << 20)  # the entry point's own capacity arithmetic
    first = np.concatenate([np.arange(n, dtype=np.int64), [n - 1]])
    head = np.arange(1, n, dtype=np.int32)
    parent = np.concatenate([np.arange(1, n, dtype=np.int64), [-1]])
    e_arc = np.arange(n - 1, dtype=np.int64)
    e_up = np.ones(n - 1, np.int8)
    topo = DeviceTopology(n, first, head, parent, e_arc, e_up)
    # the call is rejected before any launch, so the arcs need no values
    up = torch.zeros(n - 1, dtype=torch.int32, device="cuda")
    noalloc = _bind(_lib.lib())
    s_dev = torch.zeros(4, dtype=torch.int32, device="cuda")
    out = torch.full((4,), -7, dtype=torch.int64, device="cuda")
    rc = noalloc(topo.handle, up.data_ptr(), up.data_ptr(), s_dev.data_ptr(), s_dev.data_ptr(), 4,
                 out.data_ptr(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -7  # NWCCH_ERR_CAPACITY
    assert (out.cpu().numpy() == -7).all()  # nothing was launched

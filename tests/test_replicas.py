"""Multi-GPU host logic on CPU: bench.py's replica path (one replica per rank,
no data-path collective, the maximum time over ranks) run on two gloo ranks.
Every rank customizes its own replica of the same metric with the oracle; the
replicas agree bit for bit and the timing reduction is the maximum."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import numpy as np
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    sys.path[:0] = [str(ROOT), str(ROOT / "oracle"), str(ROOT / "negative-weight-cch_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle as orc
        from nwcch import graphs as G
        from nwcch import topology as TT
        g = G.grid(24, seed=4)
        top = TT.build_topology(g, leaf=16)
        OT = orc.Topo.from_dict(top)
        up, dn = orc.customize(OT, g["w"])
        digest = float(np.bitwise_xor.reduce(up[up != orc.INF] * 31 + dn[dn != orc.INF]))
        gathered = [None] * world
        dist.all_gather_object(gathered, digest)
        t = bench.max_over_ranks([1.0 + rank, 10.0 * (world - rank)], "cpu")
        out.put((rank, gathered, t, bench.replica_units(5, world)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, t, units in res:
        assert gathered[0] == gathered[1]   # replicas agree
        assert t == [2.0, 20.0]             # maximum over ranks, element-wise
        assert units == 10

"""Replica sharding across ranks (bench.py --gpus N), on CPU with gloo.

Each rank solves its own shard of queries on its own PCG32 streams
(bench.shard); two ranks together must reproduce one single-process run of
the combined queries exactly, and the timing reduction takes the maximum over
ranks (bench.max_over_ranks).  The solver here is the CPU oracle: the test
covers the host-side sharding logic, which is identical for the GPU library.
"""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
N = 48


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from conftest import load_package
    load_package()
    from sms_gb300 import workloads as W
    from oracle import oracle as O
    first, offset = bench.shard(rank, N)
    q = W.water_queries(N, first=first)
    v, c, w, _ = O.OracleScene(W.water_scene(res=32)).connect_batch(W.water_config(), q, seed=7,
                                                                    stream_offset=offset, nthreads=1)
    parts = [None] * world
    dist.all_gather_object(parts, (rank, v, c, w))
    mx = bench.max_over_ranks(torch, [float(rank + 1), 10.0 - rank], "cpu")
    if rank == 0:
        out.put((parts, mx))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_reproduce_single_run():
    import torch.multiprocessing as mp
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    O.load()   # build the oracle before the ranks start
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    parts, mx = out.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert mx == [2.0, 10.0]
    parts = sorted(parts, key=lambda t: t[0])
    v = np.concatenate([t[1] for t in parts], axis=1)
    c = np.concatenate([t[2] for t in parts])
    w = np.concatenate([t[3] for t in parts])
    sys.path.insert(0, str(ROOT / "tests"))
    from conftest import load_package
    load_package()
    from sms_gb300 import workloads as W
    q = W.water_queries(2 * N)
    vs, cs, ws, _ = O.OracleScene(W.water_scene(res=32)).connect_batch(W.water_config(), q, seed=7, nthreads=1)
    np.testing.assert_array_equal(v, vs)
    np.testing.assert_array_equal(c, cs)
    np.testing.assert_array_equal(w, ws)
    assert ws.sum() > 2 * N   # some queries ran Bernoulli trials

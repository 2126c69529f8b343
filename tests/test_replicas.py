"""Replica sharding across ranks (CPU, gloo, world size 2)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import load_pkg


def test_shard_partitions_exactly():
    load_pkg()
    from mlem_gb300.replicas import shard
    for count in (0, 1, 7, 64, 101):
        for world in (1, 2, 3, 8):
            parts = [shard(count, r, world) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(count))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.environ["MLEM_TEST_ROOT"])
    from conftest import load_pkg
    load_pkg()
    from mlem_gb300.replicas import run_sharded
    from oracle import oracle as O
    # each instance: a tiny reconstruction on the CPU oracle (the checker stands
    # in for the per-rank GPU so the host logic is exercised without a GPU)
    rng = np.random.Generator(np.random.PCG64(0))
    rows, cols = 40, 12
    rp = np.arange(0, rows * 3 + 1, 3, dtype=np.uint64)
    col = rng.integers(0, cols, rows * 3).astype(np.uint32)
    val = rng.uniform(0.1, 1, rows * 3).astype(np.float32)
    norm = O.colsum(rp, col, val, cols)
    def fn(i):
        g = np.random.Generator(np.random.PCG64(100 + i)).integers(0, 50, rows).astype(np.int32)
        return O.mlem_f64((rp, col, val), g, norm, np.ones(cols), 5)
    out = run_sharded(fn, 9)
    if rank == 0:
        q.put([o.tolist() for o in out])
    dist.destroy_process_group()


def test_run_sharded_gathers_in_order(tmp_path):
    from conftest import ROOT
    os.environ["MLEM_TEST_ROOT"] = str(ROOT)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import sys
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    rng = np.random.Generator(np.random.PCG64(0))
    rows, cols = 40, 12
    rp = np.arange(0, rows * 3 + 1, 3, dtype=np.uint64)
    col = rng.integers(0, cols, rows * 3).astype(np.uint32)
    val = rng.uniform(0.1, 1, rows * 3).astype(np.float32)
    norm = O.colsum(rp, col, val, cols)
    for i in range(9):
        g = np.random.Generator(np.random.PCG64(100 + i)).integers(0, 50, rows).astype(np.int32)
        assert np.allclose(res[i], O.mlem_f64((rp, col, val), g, norm, np.ones(cols), 5), rtol=0, atol=0)

"""The multi-rank host logic on CPU with 2 gloo ranks: sharded sources, one
all-reduce of the BC partials and a gather of closeness sums reproduce the
single-rank result (partials computed by the oracle on CPU)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from bc_gb300.shard import combine_bc, gather_cc, shard_sources
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(1)
    n = 600
    row = np.zeros(n + 1, np.int64)
    adj = [set() for _ in range(n)]
    for _ in range(2400):
        u, v = rng.integers(0, n, 2)
        if u != v:
            adj[u].add(int(v))
            adj[v].add(int(u))
    col = []
    for v in range(n):
        row[v + 1] = row[v] + len(adj[v])
        col += sorted(adj[v])
    g = O.Graph(row, np.array(col, np.int32))
    src = rng.integers(0, n, 333).astype(np.int32)
    mine = shard_sources(src, rank, world, batch=64)
    part, _ = O.bc(g, mine) if len(mine) else (np.zeros(n), 0)
    total = combine_bc(part)
    cc = gather_cc(O.cc(g, mine))
    if rank == 0:
        np.save(os.path.join(out_dir, "bc.npy"), total)
        np.save(os.path.join(out_dir, "cc.npy"), cc)
        order = np.concatenate([shard_sources(src, r, world, batch=64) for r in range(world)])
        np.save(os.path.join(out_dir, "order.npy"), order)
        full, _ = O.bc(g, src)
        np.save(os.path.join(out_dir, "bc_full.npy"), full)
        np.save(os.path.join(out_dir, "cc_full.npy"), O.cc(g, order))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shard_and_combine(tmp_path, orc):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    bc = np.load(tmp_path / "bc.npy")
    full = np.load(tmp_path / "bc_full.npy")
    assert np.max(np.abs(bc - full) / np.maximum(np.abs(full), 1.0)) < 1e-12
    assert np.array_equal(np.load(tmp_path / "cc.npy"), np.load(tmp_path / "cc_full.npy"))


def test_shard_sources_partition():
    from bc_gb300.shard import shard_sources
    s = np.arange(1000, dtype=np.int32)
    for world in (1, 2, 3, 8):
        for batch in (0, 64):
            parts = [shard_sources(s, r, world, batch) for r in range(world)]
            assert np.array_equal(np.sort(np.concatenate(parts)), s)
    with pytest.raises(ValueError):
        shard_sources(s, 2, 2)

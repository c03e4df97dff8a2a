"""Host-side multi-rank logic for the batched path: sources are independent,
so ranks take disjoint shares of the source list (no data-path collective);
a full betweenness vector is the sum of the per-rank partials, combined with
one all-reduce at the end.  Closeness sums need only a gather."""
from __future__ import annotations

import numpy as np


def shard_sources(sources, rank: int, world: int, batch: int = 0) -> np.ndarray:
    """Rank `rank`'s share of `sources`.  With batch > 0 the list is dealt in
    whole batches round-robin (batch i goes to rank i % world), so every rank
    runs full lane batches; otherwise contiguous near-equal slices."""
    s = np.ascontiguousarray(sources, dtype=np.int32)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    if batch > 0:
        nb = (len(s) + batch - 1) // batch
        idx = [np.arange(b * batch, min((b + 1) * batch, len(s))) for b in range(rank, nb, world)]
        return s[np.concatenate(idx)] if idx else s[:0]
    lo = len(s) * rank // world
    hi = len(s) * (rank + 1) // world
    return s[lo:hi]


def combine_bc(bc_partial: np.ndarray, group=None) -> np.ndarray:
    """Sum of the ranks' FP64 betweenness partials (torch.distributed all-reduce)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(bc_partial, dtype=np.float64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def gather_cc(cc_partial: np.ndarray, group=None) -> np.ndarray:
    """Concatenation, in rank order, of the ranks' closeness sums."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"   # NCCL gathers device tensors only
    n = torch.tensor([len(cc_partial)], dtype=torch.int64, device=dev)
    sizes = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    mx = int(max(x.item() for x in sizes))
    buf = torch.zeros(mx, dtype=torch.int64, device=dev)
    buf[:len(cc_partial)] = torch.from_numpy(np.ascontiguousarray(cc_partial, dtype=np.int64)).to(dev)
    out = [torch.zeros(mx, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(out, buf, group=group)
    return np.concatenate([o[:int(s.item())].cpu().numpy() for o, s in zip(out, sizes)])

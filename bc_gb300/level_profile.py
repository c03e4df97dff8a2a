"""Per-level profile of one lane batch: frontier entries and device time per
BFS level, forward and dependency sweep, binned into level ranges.

    python -m bc_gb300.level_profile grid 1024 [--sources 1024] [--bins 16]
    python -m bc_gb300.level_profile rmat 22

Runs one betweenness batch with one level kernel per captured graph
(levels_per_graph = 1), so each graph launch's CUDA-event time is one level's.
Prints one JSON object: the graph, settings, totals and per-bin rows of
(levels, entries, forward ms, sweep ms, entries per microsecond).
"""
from __future__ import annotations

import argparse
import json

import numpy as np

import bc_gb300 as G


def make(kind: str, size: int):
    if kind == "grid":
        return G.gen_grid(size, size, 0.05, seed=3, largest_only=True), f"grid{size}_minus5pct_largest"
    return G.gen_rmat(size, 16, seed=1, permute=True), f"rmat{size}_ef16"


def profile(csr, sources, lanes, group, block, bins):
    with G.Graph(csr) as g:
        opt = dict(lanes=lanes, group_lanes=group, levels_per_graph=1, delta_precision=G.DELTA_F32,
                   block_threads=block)
        g.bc(sources, **opt)          # warm-up: level width, queue size, graph capture
        g.bc(sources, **opt)
        st = g.stats()
        lv = g.levels()
    ent, fw, bw = lv["entries"], lv["fwd_ms"], lv["bwd_ms"]
    L = len(ent)
    # forward launch i runs level i; the sweep runs levels L-1 .. 1, launch j -> level L-1-j
    fwd = np.zeros(L)
    fwd[: min(L, len(fw))] = fw[:L]
    bwd = np.zeros(L)
    for j, ms in enumerate(bw):
        if L - 1 - j >= 1:
            bwd[L - 1 - j] = ms
    edges = np.linspace(0, L, bins + 1).astype(int)
    rows = []
    for a, b in zip(edges[:-1], edges[1:]):
        if b <= a:
            continue
        e = int(ent[a:b].sum())
        f, w = float(fwd[a:b].sum()), float(bwd[a:b].sum())
        rows.append({"levels": [int(a), int(b - 1)], "entries": e, "fwd_ms": round(f, 3), "bwd_ms": round(w, 3),
                     "fwd_entries_per_us": round(e / max(f, 1e-9) / 1e3, 1),
                     "us_per_fwd_level": round(f * 1e3 / (b - a), 1)})
    return {"levels": L, "entries": int(ent.sum()), "fwd_ms": round(float(fwd.sum()), 3),
            "bwd_ms": round(float(bwd.sum()), 3), "sigma_mode_used": st["sigma_mode_used"],
            "group_lanes": st["group_lanes"], "lanes": st["lanes"], "bins": rows}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("kind", choices=["grid", "rmat"])
    p.add_argument("size", type=int, help="grid side, or R-MAT scale")
    p.add_argument("--sources", type=int, default=1024)
    p.add_argument("--lanes", type=int, default=1024)
    p.add_argument("--group", type=int, default=0, choices=(0, 1, 32, 128))
    p.add_argument("--block", type=int, default=0, choices=(0, 128, 256, 512))
    p.add_argument("--bins", type=int, default=16)
    a = p.parse_args()
    csr, name = make(a.kind, a.size)
    cand = np.nonzero(np.diff(csr.row) > 0)[0].astype(np.int32)
    src = cand[np.random.default_rng(4).integers(0, len(cand), size=a.sources)].astype(np.int32)
    out = {"graph": name, "n": csr.n, "m": int(csr.m) // 2, "sources": a.sources}
    out.update(profile(csr, src, a.lanes, a.group, a.block, a.bins))
    print(json.dumps(out))


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Throughput of batched Brandes betweenness on one GB300 (GTEPS).

Workload: R-MAT scale 22, edge factor 16 (a=.57, b=.19, c=.19; symmetrised,
self-loops and duplicates dropped; seeded vertex relabelling), k = 16,384
sampled sources (seed 4, uniform over vertices with at least one edge).  A
step is one lane batch: `--lanes` sources (default 1024) run forward BFS with
exact uint64 path counts and the dependency sweep, accumulating FP64 BC.
GTEPS = sum over the step's sources of the undirected edges of the source's
component / time.

  value : device-resident inputs, gbc_bc_device on a resident graph, CUDA
          events on the launching stream over exactly --steps steps.
  e2e   : the host-buffer C ABI a drop-in caller uses -- per step the CSR and
          the sources are copied from pinned host memory (gbc_graph_create +
          gbc_bc) and the BC vector is read back.
  plain : the one-source-at-a-time engine on a sample of the same sources.
  roofline : the dominant level kernel's algorithmic bytes per launch (adjacency
          once + 16 B per lane and vertex of lane state per sweep, + 16 B per
          vertex of BC accumulation in the sweep) over its CUDA-event duration,
          against the measured HBM copy bandwidth; traffic from the committed
          ncu summary (a small-case capture scaled by those bytes);
          visit_model: the bytes the kernels request (own level row and lane
          state per frontier entry, the neighbour's level row per neighbour
          visit, one path count / rho per lane and undirected edge).
  cpu_baseline : the oracle's FP64 Brandes with all host threads on a
          bounded sample of the same sources.
  clocks : SM clocks and throttle reasons sampled during the timed region.
  serving : the serving mix over 64 resident graphs (rates, saturation), and
          bench_graph: k=1024 / k=64 sampled-BC queries served on the R-MAT
          s22 graph itself, delivered GTEPS beside the plain engine's.
  ba_all_sources / reduction / deep_grid : the other single-GPU
          configurations in short form -- BA n=4096 m=4 with every vertex a
          source (FP64 delta betweenness and closeness, with rooflines); the
          D1+AP reduction on R-MAT s18 + 60K pendant trees and on the same
          R-MAT with 30K attached cycles (device reduction, reduced vs
          unreduced closeness and betweenness); the 1024^2 grid with 8,192
          autotuned sources (wide path counts, with rooflines).

--impl reference times the CPU restatement of the reference's sequential
Brandes (oracle/, the reference's own code is not buildable on the GPU host)
with all host threads, on a bounded sample of the same sources per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BC/CC GTEPS & p50/p99 query latency, batched+served vs plain, 1×GB300"
WORKLOAD = "rmat22_ef16_sampled_bc_k16384"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=4)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--lanes", type=int, default=1024)
    p.add_argument("--scale", type=int, default=22)
    p.add_argument("--edge-factor", type=int, default=16)
    p.add_argument("--k", type=int, default=16384)
    p.add_argument("--delta", default="f32", choices=["f32", "f64"],
                   help="dependency-sweep precision (FP32 delta with FP64 BC sums is the default design)")
    p.add_argument("--plain-sources", type=int, default=16)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-tune", action="store_true", help="skip gbc_autotune; use the default expansion settings")
    p.add_argument("--group-lanes", type=int, default=0, choices=(0, 32, 128),
                   help="sources per lane group (0: the library's choice)")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=5.0, help="arrival window per rate")
    p.add_argument("--serve-rates", default="5,10,20,40", help="query arrival rates per second, comma-separated")
    p.add_argument("--serve-burst", type=int, default=96, help="queries submitted at once for the saturation point")
    p.add_argument("--serve-workers", type=int, default=0, help="server worker threads (0: the library default, 8)")
    p.add_argument("--no-serve", action="store_true")
    p.add_argument("--serve-graph-rate", type=float, default=6.0,
                   help="query arrival rate of the serving stream on the benchmark graph itself")
    p.add_argument("--serve-graph-burst", type=int, default=32,
                   help="queries submitted at once on the benchmark graph (0: none)")
    p.add_argument("--no-reduction", action="store_true", help="skip the D1+AP reduction section (R-MAT s18 + pendant trees)")
    p.add_argument("--no-grid", action="store_true", help="skip the deep-grid section (1024^2 grid, 8192 sources)")
    p.add_argument("--grid-sources", type=int, default=8192, help="sources of the deep-grid section")
    p.add_argument("--no-ba", action="store_true", help="skip the all-sources section (BA n=4096, m=4)")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def sample_sources(row, k):
    """k sources, uniform (seed 4) over the vertices with at least one edge."""
    cand = np.nonzero(np.diff(row) > 0)[0].astype(np.int32)
    rng = np.random.default_rng(4)
    return cand[rng.integers(0, len(cand), size=k)].astype(np.int32)


def make_graph(args):
    """The workload graph from the product's generator (GPU arm)."""
    import bc_gb300 as G
    csr = G.gen_rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=1, permute=True)
    return csr, sample_sources(csr.row, args.k)


def make_graph_oracle(args):
    """The same graph from the oracle's restatement of that generator (CPU
    legs: the reference arm never loads the product library); identical
    arrays, checked in tests/test_oracle.py."""
    from oracle import oracle as O
    g = O.gen_rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=1, permute=True)
    return g, sample_sources(g.row, args.k)


def comp_edges(csr):
    """Undirected edges of each vertex's component (GTEPS numerator)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    n = len(csr.row) - 1
    A = sp.csr_matrix((np.ones(len(csr.col), np.int8), csr.col, csr.row), shape=(n, n))
    nc, lab = connected_components(A, directed=False)
    e = np.bincount(lab, weights=np.diff(csr.row), minlength=nc) / 2
    return e[lab].astype(np.int64)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_traffic():
    """Per-launch DRAM traffic of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_summary.json")
    if not os.path.exists(p):
        return None
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def cpu_baseline(csr, sample, n_src, threads):
    """Oracle (CPU restatement of Seq_Brandes/Brandes.c:224) on a bounded sample."""
    from oracle import oracle as O
    og = O.Graph(csr.row, csr.col)
    src = sample[:n_src]
    t = time.perf_counter()
    O.bc(og, src, semantics=O.BC_REFERENCE, nthreads=threads)
    dt = time.perf_counter() - t
    return dt


def server_counters(G, L, h):
    import ctypes as C
    v = [C.c_int64() for _ in range(4)] + [C.c_double()]
    G.check(L.gbc_server_counters(h, *[C.byref(x) for x in v]))
    return [x.value for x in v]


def serve_stream(G, L, h, draw, n_of, rate, seconds, count, rng):
    """One arrival stream on a server: `count` queries at once (a burst), or
    Poisson arrivals at `rate` per second for `seconds`.  Every query is waited
    for and fetched; latencies are the server's submit-to-completion times.
    draw() submits one query and returns (request id, graph index)."""
    import ctypes as C
    c0 = server_counters(G, L, h)
    t0 = time.perf_counter()
    t_end = t0 + seconds
    reqs = [draw() for _ in range(count)] if count else []
    while not count and time.perf_counter() < t_end:
        reqs.append(draw())
        time.sleep(rng.expovariate(rate))
    lats = []
    for rid, gi in reqs:
        st = C.c_int32()
        G.check(L.gbc_server_wait(h, rid, 600000.0, C.byref(st)))
        n = n_of(gi)
        bc = np.zeros(n)
        cc = np.zeros(n, np.int64)
        lat = C.c_double()
        G.check(L.gbc_server_fetch(h, rid, bc.ctypes.data_as(C.c_void_p), cc.ctypes.data_as(C.c_void_p),
                                   C.byref(lat)))
        lats.append(lat.value)
    wall = time.perf_counter() - t0
    c1 = server_counters(G, L, h)
    lats = np.array(lats)
    busy = c1[4] - c0[4]
    return {"rate_per_s": rate if not count else "burst", "queries": len(lats),
            "p50_ms": round(float(np.percentile(lats, 50)), 3),
            "p99_ms": round(float(np.percentile(lats, 99)), 3), "wall_s": round(wall, 3),
            "lane_batches": c1[1] - c0[1], "shared_batches": c1[2] - c0[2],
            "gteps_delivered": round((c1[3] - c0[3]) / wall / 1e9, 3),
            "busy_frac": round(busy * 1e-3 / wall, 3)}


def serving(G, seconds, rates, burst=96, seed=11, workers=0):
    """The serving mix: a Poisson stream of queries over 64 device-resident
    graphs of 1K-2M vertices (BA m=2-8, Erdos-Renyi average degree 4-32,
    square grids, R-MAT scale 10-21; seeded sizes, log-uniform).  Queries:
    exact CC and exact BC on the smaller graphs, k = 64 / 1024 sampled BC
    everywhere.  One stream per arrival rate, on the same server; per rate the
    p50/p99 latency and the GTEPS delivered over the stream's wall time
    (first arrival to last completion).  The saturation point submits `burst`
    queries of the same mix at once: its delivered GTEPS is the server's
    capacity on this mix (the GPU busy nearly all of the time)."""
    import ctypes as C
    import random
    L = G.lib()
    grng = np.random.default_rng(5)
    specs = []
    for i in range(64):
        n = int(np.exp(grng.uniform(np.log(1000), np.log(2_000_000))))
        fam = i % 4
        if fam == 0:
            specs.append(("ba", G.gen_ba(n, int(grng.integers(2, 9)), i)))
        elif fam == 1:
            specs.append(("er", G.gen_er(n, float(grng.uniform(4, 32)), i)))
        elif fam == 2:
            side = max(8, int(np.sqrt(n)))
            specs.append(("grid", G.gen_grid(side, side, 0.0, i)))
        else:
            specs.append(("rmat", G.gen_rmat(int(np.clip(round(np.log2(n)), 10, 21)), 16, seed=i)))
    cfg = G.ServerConfig()
    cfg.max_lanes = 1024
    cfg.workers = workers
    h = C.c_void_p()
    G.check(L.gbc_server_create(C.byref(cfg), C.byref(h)))
    gids = []
    for _, csr in specs:
        gid = C.c_int32()
        G.check(L.gbc_server_add_graph(h, csr.row, csr.col, csr.n, C.byref(gid)))
        gids.append(gid.value)
    rng = random.Random(seed)
    o = G.options()

    def draw():
        gi = rng.randrange(len(specs))
        n = specs[gi][1].n
        r = rng.random()
        if r < 0.15 and n <= 32768:
            kind, k = G.Q_CC, 0
        elif r < 0.25 and n <= 16384:
            kind, k = G.Q_BC, 0
        elif r < 0.65:
            kind, k = G.Q_BC_SAMPLED, 64
        else:
            kind, k = G.Q_BC_SAMPLED, 1024
        rid = C.c_int64()
        G.check(L.gbc_server_submit(h, gids[gi], kind, k, rng.randrange(1 << 30), C.byref(o), 0.0, C.byref(rid)))
        return rid.value, gi

    def n_of(gi):
        return specs[gi][1].n

    points = [serve_stream(G, L, h, draw, n_of, r, seconds, 0, rng) for r in rates]
    sat = serve_stream(G, L, h, draw, n_of, 0.0, seconds, burst, rng) if burst else None
    L.gbc_server_destroy(h)
    return {"graphs": len(specs), "vertices": [min(c.n for _, c in specs), max(c.n for _, c in specs)],
            "directed_entries": int(sum(c.m for _, c in specs)), "workers": workers or 8, "points": points,
            "saturation": sat,
            "mix": "uniform over graphs: 15% exact CC (graphs <= 32K vertices), 10% exact BC (<= 16K), "
                   "40% k=64 and 35% k=1024 sampled BC"}


def served_bench_graph(G, csr, seconds, rate, burst, plain_gteps, seed=23, workers=0):
    """Serving on the benchmark graph itself (R-MAT s22 ef16, resident on a
    server): sampled-BC queries of k = 1024 and k = 64 sources (half each,
    drawn by the server uniformly over all vertices with the query's seed;
    FP32 delta, Brandes semantics), first as a Poisson stream at `rate` per
    second for `seconds`, then `burst` queries at once.  Delivered GTEPS is
    the edges of the sources' components over the stream's wall time, set
    beside the one-source-at-a-time engine's GTEPS on the same graph."""
    import ctypes as C
    import random
    L = G.lib()
    cfg = G.ServerConfig()
    cfg.max_lanes = 1024
    cfg.workers = workers
    h = C.c_void_p()
    G.check(L.gbc_server_create(C.byref(cfg), C.byref(h)))
    gid = C.c_int32()
    t0 = time.perf_counter()
    G.check(L.gbc_server_add_graph(h, csr.row, csr.col, csr.n, C.byref(gid)))
    add_s = time.perf_counter() - t0
    rng = random.Random(seed)
    o = G.options(delta_precision=G.DELTA_F32)

    def draw():
        k = 1024 if rng.random() < 0.5 else 64
        rid = C.c_int64()
        G.check(L.gbc_server_submit(h, gid.value, G.Q_BC_SAMPLED, k, rng.randrange(1 << 30), C.byref(o), 0.0,
                                    C.byref(rid)))
        return rid.value, 0

    points = [serve_stream(G, L, h, draw, lambda gi: csr.n, rate, seconds, 0, rng)]
    if burst:
        points.append(serve_stream(G, L, h, draw, lambda gi: csr.n, 0.0, seconds, burst, rng))
    L.gbc_server_destroy(h)
    best = max(p["gteps_delivered"] for p in points)
    return {"graph": "rmat22_ef16", "add_graph_s": round(add_s, 3), "queries": "50% k=1024, 50% k=64 sampled BC",
            "points": points, "gteps_delivered_best": best,
            "speedup_vs_plain": None if not plain_gteps else round(best / plain_gteps, 2)}


def kernel_roofline(st, n, M, k, job, hbm, peak_kind):
    """Roofline of the dominant level kernel of one library call, from its
    statistics (CUDA-event device time of the forward and dependency-sweep
    level launches).  Algorithmic bytes per lane batch of B sources:
    betweenness, per sweep, adjacency once (4 M + 4 (n + 1)) + 16 B n of lane
    state, + 16 n of BC accumulation in the sweep; closeness, adjacency once
    + B n / 4 (a visited and a frontier bit per lane, written and read) + 8 B."""
    batches = max(int(st["batches"]), 1)
    adj = 4 * M + 4 * (n + 1)
    if job == "bc":
        fwd = batches * adj + 16 * k * n
        bwd = batches * (adj + 16 * n) + 16 * k * n
        if st["fwd_ms"] >= st["bwd_ms"]:
            name, ms, nb, launches = "forward", st["fwd_ms"], fwd, st["fwd_kernels"]
        else:
            name, ms, nb, launches = "sweep", st["bwd_ms"], bwd, st["bwd_kernels"]
    else:
        name, ms, nb, launches = "forward", st["fwd_ms"], batches * adj + k * n // 4 + 8 * k, st["fwd_kernels"]
    ach = nb / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    return {"bound": "hbm", "levels": name, "achieved": round(ach, 2), "peak": hbm, "unit": "GB/s",
            "frac": round(ach / hbm, 5), "traffic": None, "peak_kind": peak_kind,
            "alg_bytes_per_launch": int(nb / max(launches, 1)), "avg_launch_ms": round(ms / max(launches, 1), 4),
            "kernel": ("expand" if name == "forward" else "backward")
                      + {128: "_q", 1: "_s"}.get(int(st["group_lanes"]), "") + "_kernel"}


def ba_section(G, hbm, peak_kind):
    """The plain exact configuration: Barabasi-Albert n = 4096, m = 4, seed 1,
    every vertex a source, betweenness with FP64 delta and closeness; GTEPS
    and roofline from the library's CUDA-event timing (best of three calls)."""
    csr = G.gen_ba(4096, 4, 1)
    out = {"graph": "ba4096_m4_seed1", "n": int(csr.n), "m": int(csr.m // 2), "sources": int(csr.n)}
    with G.Graph(csr) as g:
        for job in ("bc", "cc"):
            best = None
            for _ in range(3):
                if job == "bc":
                    g.bc(None, delta_precision=G.DELTA_F64)
                else:
                    g.cc(None)
                st = g.stats()
                if best is None or st["kernel_ms"] < best["kernel_ms"]:
                    best = st
            out[job] = {"gteps": round(best["edges_traversed"] / best["kernel_ms"] / 1e6, 3),
                        "ms": round(best["kernel_ms"], 3), "lanes": int(best["lanes"]),
                        "roofline": kernel_roofline(best, csr.n, csr.m, csr.n, job, hbm, peak_kind)}
        # source order: the library's level-profile grouping (above) against the reference's
        # shared-BFS pairing (Brandes.c:417-475, each source followed by its first neighbour of
        # degree != 1 not yet done) and plain id order, both kept as given (source_order = 1)
        orders = {"pairing": pairing_order(csr), "id": np.arange(csr.n, dtype=np.int32)}
        for name, order in orders.items():
            best = None
            for _ in range(3):
                g.bc(order, delta_precision=G.DELTA_F64, source_order=1)
                st = g.stats()
                best = st["kernel_ms"] if best is None else min(best, st["kernel_ms"])
            out["bc"]["ms_" + name + "_order"] = round(best, 3)
    return out


def pairing_order(csr):
    """The reference shared-BFS driver's source sequence: in id order, each
    source not yet done, then its first neighbour of degree != 1 not yet done."""
    deg = np.diff(csr.row)
    done = np.zeros(csr.n, bool)
    out = []
    for s in range(csr.n):
        if done[s]:
            continue
        done[s] = True
        out.append(s)
        for x in csr.col[csr.row[s]:csr.row[s + 1]]:
            if deg[x] != 1 and not done[x]:
                done[x] = True
                out.append(int(x))
                break
    return np.array(out, np.int32)


def reduction_section(G):
    """The D1-folding + articulation-point configurations: R-MAT scale 18,
    edge factor 4, with 60K pendant trees of depth 1-3 (382K vertex slots;
    its folded 2-core has no articulation point), and the same R-MAT with 30K
    cycles of 3-6 vertices and 60K pendant trees attached (articulation points
    with small blocks behind them).  Device reduction, then closeness and
    betweenness of every vertex through it against the unreduced graph (wall
    times of the calls, device-resident)."""
    G.Reduced(G.add_pendants(G.gen_rmat(10, 4, seed=1), 100, 3, 2))   # first-call setup

    def wall(f):
        t = time.perf_counter()
        r = f()
        return r, (time.perf_counter() - t) * 1e3

    def one(name, csr):
        R, t_red = wall(lambda: G.Reduced(csr))
        info = R.info()
        cc_r, t_ccr = wall(R.cc)
        bc_r, t_bcr = wall(R.bc)
        R.close()
        with G.Graph(csr) as g:
            cc_p, t_ccp = wall(g.cc)
            bc_p, t_bcp = wall(g.bc)
        rel = float(np.max(np.abs(bc_r - bc_p) / np.maximum(np.abs(bc_p), 1.0)))
        return {"graph": name, "n": int(csr.n), "m": int(csr.m // 2),
                "reduce_ms": round(t_red, 2), "folded": info["d1_folded"], "fold_rounds": info["fold_rounds"],
                "articulation_points": info["articulation_points"], "blocks": info["blocks"],
                "max_block": info["max_block"], "block_slots": info["block_slots"],
                "cc_reduced_ms": round(t_ccr, 1), "cc_unreduced_ms": round(t_ccp, 1),
                "cc_bit_equal": bool(np.array_equal(cc_r, cc_p)),
                "bc_reduced_ms": round(t_bcr, 1), "bc_unreduced_ms": round(t_bcp, 1), "bc_max_rel_diff": rel}

    base = G.gen_rmat(18, 4, seed=18)
    out = one("rmat18_ef4+60k_pendant_trees", G.add_pendants(base, 60000, 3, 2))
    out["with_articulation_points"] = one("rmat18_ef4+30k_cycles_3to6+60k_pendant_trees",
                                          G.add_pendants(G.add_cycles(base, 30000, 3, 6, 5), 60000, 3, 2))
    return out


def grid_section(G, hbm, peak_kind, k=8192):
    """The deep configuration: 1024 x 1024 grid with 5% of the edges removed
    (seed 3), largest component, k = 8,192 uniformly sampled sources (seed
    3): autotuned batches, betweenness (FP32 delta; path counts pass 2^64, so
    wide form) and closeness, GTEPS and roofline from the library's own
    CUDA-event timing."""
    grid = G.gen_grid(1024, 1024, 0.05, seed=3, largest_only=True)
    src = np.random.default_rng(3).choice(grid.n, 8192, replace=False).astype(np.int32)[:k]
    with G.Graph(grid) as g:
        t = time.perf_counter()
        tuning = g.autotune(src, delta_precision=G.DELTA_F32)
        t_tune = time.perf_counter() - t
        g.bc(src, delta_precision=G.DELTA_F32)
        st = g.stats()
        g.cc(src)
        st2 = g.stats()
    return {"graph": "grid1024_minus5pct_largest", "n": int(grid.n), "m": int(grid.m // 2), "sources": int(k),
            "tuning": tuning, "autotune_s": round(t_tune, 2),
            "bc_gteps": round(st["edges_traversed"] / st["kernel_ms"] / 1e6, 3), "bc_ms": round(st["kernel_ms"], 1),
            "bc_levels": int(st["levels"]), "batches": int(st["batches"]),
            "sigma_mode": "wide" if st["sigma_mode_used"] == G.SIGMA_WIDE else "exact",
            "lanes": int(st["lanes"]), "lanes_per_group": int(st["group_lanes"]),
            "bc_roofline": kernel_roofline(st, grid.n, grid.m, k, "bc", hbm, peak_kind),
            "cc_gteps": round(st2["edges_traversed"] / st2["kernel_ms"] / 1e6, 3), "cc_ms": round(st2["kernel_ms"], 1),
            "cc_roofline": kernel_roofline(st2, grid.n, grid.m, k, "cc", hbm, peak_kind)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    csr, sample = make_graph_oracle(args)
    ce = comp_edges(csr)
    threads = os.cpu_count() or 1
    n_src = max(threads, 8)
    # warm-up (page-in) and timed steps: each step a bounded slice of the sample
    times, edges = [], 0
    for i in range(args.warmup + args.steps):
        lo = (i * n_src) % len(sample)
        src = sample[lo:lo + n_src]
        dt = cpu_baseline(csr, src, len(src), threads)
        if i >= args.warmup:
            times.append(dt)
            edges += int(ce[src].sum())
    tot = sum(times)
    gteps = edges / tot / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": round(gteps, 6), "unit": "GTEPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * tot / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded R-MAT generator)",
            "config": {"workload": WORKLOAD, "scale": args.scale, "edge_factor": args.edge_factor,
                       "n": int(len(csr.row) - 1), "m_directed": int(csr.row[-1]), "sources": args.k,
                       "sources_per_step": n_src,
                       "why_fewer_sources_per_step": (
                           f"a step here is {n_src} of the same sampled sources, not a 1024-lane batch: the CPU port "
                           "runs ~0.24 GTEPS on 16 host threads, so a 1024-source step would take ~4.5 min; GTEPS is "
                           "a rate over the same graph and sample"),
                       "graph_builder": "oracle restatement of the seeded R-MAT generator (libgbc not loaded)"},
            "cpu_baseline": {"value": round(gteps, 6), "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"{n_src} sampled sources per step (reference semantics, FP64)"},
            "e2e": {"value": round(gteps, 6), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import ctypes as C

    import torch

    import bc_gb300 as G

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    G.check(G.lib().gbc_set_device(dev.index))   # the library's own (static) CUDA runtime

    csr, sample = make_graph(args)
    ce = comp_edges(csr)
    B = args.lanes
    # weak scaling: every rank runs its own `steps` batches of distinct sources
    def step_sources(i):
        lo = ((rank * (args.warmup + args.steps) + i) * B) % len(sample)
        idx = (np.arange(B) + lo) % len(sample)
        return sample[idx]

    opt = dict(semantics=G.BC_BRANDES, delta_precision=G.DELTA_F64 if args.delta == "f64" else G.DELTA_F32,
               sigma_mode=G.SIGMA_AUTO, lanes=B, group_lanes=args.group_lanes)
    o = G.options(**opt)
    graph = G.Graph(csr)
    stream = torch.cuda.current_stream(dev)
    d_src = torch.empty(B, dtype=torch.int32, device=dev)
    d_bc = torch.empty(csr.n, dtype=torch.float64, device=dev)
    L = G.lib()

    def run_step(i):
        d_src.copy_(torch.from_numpy(step_sources(i)))
        G.check(L.gbc_bc_device(graph.h, C.c_void_p(d_src.data_ptr()), B, C.byref(o),
                                C.c_void_p(d_bc.data_ptr()), C.c_void_p(stream.cuda_stream)))
        return _stats(graph)

    def _stats(g):
        st = G.RunStats()
        G.check(L.gbc_graph_last_stats(g.h, C.byref(st)))
        return st

    # autotune the expansion settings on the first step's sources (lanes stay at B)
    tuning = None if args.no_tune else graph.autotune(step_sources(0), **opt)
    for i in range(args.warmup):
        run_step(i)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = Clocks(local)
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    fwd_ms = bwd_ms = 0.0
    fwd_k = bwd_k = launches = 0
    edges = 0
    group = 32
    visits = entries = 0
    sig_bytes = 8
    for i in range(args.warmup, args.warmup + args.steps):
        st = run_step(i)
        group = st.group_lanes
        fwd_ms += st.fwd_ms
        bwd_ms += st.bwd_ms
        fwd_k += st.fwd_kernels
        bwd_k += st.bwd_kernels
        launches += st.kernel_launches
        visits += st.neighbour_visits
        entries += st.frontier_entries
        sig_bytes = st.sigma_bytes
        edges += int(ce[step_sources(i)].sum())
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    if ws > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        te = torch.tensor([edges], device=dev, dtype=torch.float64)
        dist.all_reduce(te, op=dist.ReduceOp.SUM)
        edges_all = float(te.item())
        dist.barrier()
    else:
        edges_all = float(edges)
    gteps = edges_all / (ms * 1e-3) / 1e9

    # roofline of the dominant level kernel (algorithmic bytes per batch per sweep)
    n, M = csr.n, csr.m
    adj = 4 * M + 4 * (n + 1)
    fwd_bytes = (adj + 16 * B * n) * args.steps
    bwd_bytes = (adj + 16 * B * n + 16 * n) * args.steps
    fwd_dom = fwd_ms >= bwd_ms
    q = {128: "_q", 1: "_s"}.get(int(group), "")   # the 128-lane-group / one-lane kernels
    dom = ("expand" if fwd_dom else "backward") + q + "_kernel"
    dom_ms, dom_bytes, dom_k = (fwd_ms, fwd_bytes, fwd_k) if fwd_dom else (bwd_ms, bwd_bytes, bwd_k)
    hbm, peak_kind = peaks()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    tr = load_traffic()
    traffic = None
    if tr and dom in tr and tr[dom].get("per_launch_bytes_full_size"):
        traffic = tr[dom]["per_launch_bytes_full_size"]
    # visit model: what the level kernels request, as opposed to the lane state once per sweep.
    # Every frontier entry reads its own level row and writes its lanes' state; every neighbour
    # visit reads the neighbour's level row; each lane reads the path count (forward) or rho
    # (sweep) of each predecessor / successor, at most once per undirected edge per lane.
    row_b = group  # 8-bit levels: one byte per lane of a group
    st_b = sig_bytes if fwd_dom else 4            # FP32 rho in the default FP32-delta sweep
    vm = (entries * (row_b + group * st_b) + visits * row_b + B * (M // 2) * st_b * args.steps) / max(args.steps, 1)
    vm_launch = vm * args.steps / max(dom_k, 1)
    roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 5), "traffic": traffic, "kernel": dom, "peak_kind": peak_kind,
            "alg_bytes_per_launch": int(dom_bytes / max(dom_k, 1)),
            "avg_launch_ms": round(dom_ms / max(dom_k, 1), 4),
            "visit_model": {"bytes_per_launch": int(vm_launch),
                            "achieved": round(vm_launch / (dom_ms / max(dom_k, 1) * 1e-3) / 1e9, 2),
                            "frac": round(vm_launch / (dom_ms / max(dom_k, 1) * 1e-3) / 1e9 / hbm, 5),
                            "neighbour_visits_per_batch": int(visits / max(args.steps, 1)),
                            "frontier_entries_per_batch": int(entries / max(args.steps, 1)),
                            "path_count_bytes": sig_bytes}}

    out = None
    if rank == 0:
        # plain one-source-at-a-time engine on a sample of the same sources
        # precision: the step's sources with FP32 and FP64 dependency sweeps
        s0 = step_sources(args.warmup)
        bc32 = graph.bc(s0, **{**opt, "delta_precision": G.DELTA_F32})
        st32 = graph.stats()
        bc64 = graph.bc(s0, **{**opt, "delta_precision": G.DELTA_F64})
        st64 = graph.stats()
        nz = bc64 > 0
        prec = {"delta_f32_rel_err_vs_f64": float(np.max(np.abs(bc32 - bc64) / np.maximum(np.abs(bc64), 1.0))),
                "delta_f32_rel_err_vs_f64_nonzero": float(np.max(np.abs(bc32[nz] - bc64[nz]) / bc64[nz])) if nz.any() else 0.0,
                "gteps_f32_delta": round(st32["edges_traversed"] / (st32["kernel_ms"] * 1e-3) / 1e9, 3),
                "gteps_f64_delta": round(st64["edges_traversed"] / (st64["kernel_ms"] * 1e-3) / 1e9, 3),
                "sources": int(B),
                "note": "rel err = max|a-b|/max(|b|,1) as in the tests; the FP64-delta path is checked against the "
                        "FP64 oracle to 1e-9 in tests"}
        # closeness on the same graph: batched lanes vs the plain engine
        # (direction switching: bottom-up levels on large frontiers; the top-down-only figure beside it)
        graph.cc(s0, lanes=B, direction=1)
        stt = graph.stats()
        cc_td = float(ce[s0].sum()) / (stt["kernel_ms"] * 1e-3) / 1e9
        cc_ref = graph.cc(s0, lanes=B)
        stc = graph.stats()
        cc_gteps = float(ce[s0].sum()) / (stc["kernel_ms"] * 1e-3) / 1e9
        graph.cc(s0[:args.plain_sources], engine=G.ENGINE_PLAIN)
        stp = graph.stats()
        cc_plain = float(ce[s0[:args.plain_sources]].sum()) / (stp["kernel_ms"] * 1e-3) / 1e9
        closeness = {"value": round(cc_gteps, 3), "unit": "GTEPS", "sources": int(B),
                     "bottom_up_levels": int(stc["bottom_up_levels"]), "top_down_only": round(cc_td, 3),
                     "plain": round(cc_plain, 3), "speedup_batched_vs_plain": round(cc_gteps / cc_plain, 2)}
        plain_gteps = None
        if not args.no_plain:
            ps = sample[:args.plain_sources]
            graph.bc(ps, engine=G.ENGINE_PLAIN, **{k: v for k, v in opt.items() if k != "lanes"})
            stp = graph.stats()
            plain_gteps = float(ce[ps].sum()) / (stp["kernel_ms"] * 1e-3) / 1e9
        # e2e through the host-buffer C ABI, copies from pinned memory
        e2e = None
        if not args.no_e2e:
            row_p = torch.from_numpy(csr.row).pin_memory()
            col_p = torch.from_numpy(csr.col).pin_memory()
            bc_p = torch.empty(csr.n, dtype=torch.float64).pin_memory()
            src_p = torch.empty(B, dtype=torch.int32).pin_memory()
            row_np, col_np, bc_np, src_np = row_p.numpy(), col_p.numpy(), bc_p.numpy(), src_p.numpy()
            e2e_steps = max(1, min(args.steps, 4))
            t0 = time.perf_counter()
            e_edges = 0
            for i in range(e2e_steps):
                src_np[:] = step_sources(args.warmup + i)
                h = C.c_void_p()
                G.check(L.gbc_graph_create(row_np, col_np, csr.n, C.byref(h)))
                G.check(L.gbc_bc(h, src_np.ctypes.data_as(C.c_void_p), B, C.byref(o), bc_np))
                L.gbc_graph_destroy(h)
                e_edges += int(ce[src_np].sum())
            dt = time.perf_counter() - t0
            e2e = {"value": round(e_edges / dt / 1e9, 4), "unit": "GTEPS",
                   "h2d_bytes_per_step": int(csr.row.nbytes + csr.col.nbytes + 4 * B),
                   "d2h_bytes_per_step": int(8 * csr.n), "steps": e2e_steps,
                   "path": "gbc_graph_create + gbc_bc (host buffers)"}
        # CPU baseline: oracle on a bounded sample of the same sources
        cpu = None
        if not args.no_cpu:
            threads = os.cpu_count() or 1
            n_cpu = max(threads, 4)
            dt = cpu_baseline(csr, sample, n_cpu, threads)
            cpu = {"value": round(float(ce[sample[:n_cpu]].sum()) / dt / 1e9, 6), "unit": "GTEPS", "cores": threads,
                   "kind": "port",
                   "sample": f"first {n_cpu} of the {args.k} sampled sources, reference semantics, FP64"}
        serve = None
        if not args.no_serve:
            serve = serving(G, args.serve_seconds, [float(x) for x in args.serve_rates.split(",")], args.serve_burst,
                            workers=args.serve_workers)
            serve["bench_graph"] = served_bench_graph(G, csr, args.serve_seconds, args.serve_graph_rate,
                                                      args.serve_graph_burst, plain_gteps, workers=args.serve_workers)
        c1 = None if args.no_ba else ba_section(G, hbm, peak_kind)
        red = None if args.no_reduction else reduction_section(G)
        deep = None if args.no_grid else grid_section(G, hbm, peak_kind, args.grid_sources)
        out = {"metric": METRIC, "value": round(gteps, 4), "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "u64-sigma/" + args.delta + "-delta",
               "data": "synthetic (seeded R-MAT generator)",
               "config": {"workload": WORKLOAD, "scale": args.scale, "edge_factor": args.edge_factor,
                          "n": n, "m_directed": M, "lanes_per_step": B, "lanes_per_group": int(group), "sources": args.k,
                          "parallelism": f"sources sharded over {ws} GPU(s)",
                          "l2": "inputs larger than L2 (lane state ~16*B*n bytes per sweep)",
                          "tuning": tuning},
               "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu,
               "plain": None if plain_gteps is None else {
                   "value": round(plain_gteps, 4), "unit": "GTEPS", "sources": int(args.plain_sources),
                   "speedup_batched_vs_plain": round(gteps / plain_gteps, 2)},
               "closeness": closeness, "precision": prec, "serving": serve, "ba_all_sources": c1, "reduction": red,
               "deep_grid": deep,
               "clocks": clocks}
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    graph.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

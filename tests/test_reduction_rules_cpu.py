"""The rules of the device reduction (bc_gb300/csrc/reduce_dev.cu), restated
sequentially in Python and checked on the CPU.

  * folding in rounds: the leaves of a round are the vertices of live degree
    1 at its start; each folds into its one live neighbour, except that of two
    leaves that are each other's neighbour only the larger id folds.  Leaves are
    taken in a shuffled order, as concurrent threads would take them;
  * blocks by Tarjan-Vishkin over a BFS forest whose parents are the first
    neighbour one level up, preorder numbers with children in row order, and
    the two joining rules over tree edges.

The folded counts must equal the sequential host reduction's (gbc_reduce_host),
and the blocks and articulation points of the folded graph must equal
networkx's biconnected components on the shipped datasets and on generated
graphs with pendant trees, holes and chains of blocks.  The GPU tests compare
the device code itself with gbc_reduce_host.
"""
import numpy as np
import pytest


def _fold_rounds(row, col, n, start, rng):
    deg = np.array([row[v + 1] - row[v] if v >= start else 0 for v in range(n)])
    alive = np.array([v >= start for v in range(n)])
    cand = -np.ones(n, int)
    queue = [v for v in range(n) if v >= start and deg[v] == 1]
    folded, rnd = 0, 0
    while queue:
        for u in queue:
            if deg[u] == 1:
                cand[u] = rnd
        nxt = []
        for u in rng.permutation(queue):
            if cand[u] != rnd:
                continue
            p = next((int(col[e]) for e in range(row[u], row[u + 1]) if alive[col[e]]), -1)
            if p >= 0 and (cand[p] != rnd or u > p):
                alive[u] = False
                deg[u] = 0
                deg[p] -= 1
                folded += 1
                if deg[p] == 1:
                    nxt.append(p)
        queue, rnd = nxt, rnd + 1
    return alive, deg, folded


def _blocks(row, col, core_v, alive):
    cid = {v: i for i, v in enumerate(core_v)}
    nc = len(core_v)
    adj = [[cid[int(col[e])] for e in range(row[v], row[v + 1]) if alive[col[e]]] for v in core_v]
    uf = list(range(nc))

    def find(x):
        while uf[x] != x:
            x = uf[x]
        return x

    def union(a, b):
        a, b = find(a), find(b)
        if a != b:
            a, b = min(a, b), max(a, b)
            uf[b] = a

    for u in range(nc):
        for w in adj[u]:
            union(u, w)
    level = [0 if find(v) == v else -1 for v in range(nc)]
    levels = [[v for v in range(nc) if level[v] == 0]]
    while True:
        nxt = []
        for u in levels[-1]:
            for w in adj[u]:
                if level[w] < 0:
                    level[w] = len(levels)
                    nxt.append(w)
        if not nxt:
            break
        levels.append(nxt)
    par = [next((w for w in adj[v] if level[w] == level[v] - 1), -1) if level[v] > 0 else -1 for v in range(nc)]
    nd = [1] * nc
    for lv in reversed(levels[1:]):
        for v in lv:
            nd[par[v]] += nd[v]
    pre = [0] * nc
    for lv in levels[:-1]:
        for v in lv:
            nxt_pre = pre[v] + 1
            for w in adj[v]:
                if par[w] == v:
                    pre[w] = nxt_pre
                    nxt_pre += nd[w]
    lo, hi = list(pre), list(pre)
    for v in range(nc):
        for w in adj[v]:
            if w != par[v] and par[w] != v:
                lo[v], hi[v] = min(lo[v], pre[w]), max(hi[v], pre[w])
    for lv in reversed(levels[1:]):
        for v in lv:
            lo[par[v]], hi[par[v]] = min(lo[par[v]], lo[v]), max(hi[par[v]], hi[v])
    uf = list(range(nc))
    for u in range(nc):
        pu = par[u]
        if pu >= 0 and par[pu] >= 0 and (lo[u] < pre[pu] or hi[u] >= pre[pu] + nd[pu]):
            union(u, pu)                                   # rule (b)
        for w in adj[u]:
            if w != pu and par[w] != u and pre[w] > pre[u] and pre[w] >= pre[u] + nd[u]:
                union(u, w)                                # rule (a)
    lab = [find(v) for v in range(nc)]
    blocks, aps = {}, set()
    for v in range(nc):
        labs = {lab[v]} if par[v] >= 0 else set()
        labs |= {lab[w] for w in adj[v] if par[w] == v}
        if len(labs) >= 2:
            aps.add(core_v[v])
        if par[v] >= 0:
            blocks.setdefault(lab[v], set()).update({core_v[v], core_v[par[v]]})
        elif not adj[v]:
            blocks[("single", v)] = {core_v[v]}
    return sorted(tuple(sorted(b)) for b in blocks.values()), aps


def _graphs(gbc, datasets):
    out = {name: gbc.read_edgelist(p) for name, p in datasets.items()
           if name in ("karate.txt", "dolphins.txt", "testdata.txt", "testdata1.txt", "testdata2.txt",
                       "ia-fb-messages.mtx", "tech-WHOIS.mtx")}
    out["rmat10+pendants"] = gbc.add_pendants(gbc.gen_rmat(10, 4, seed=1), 300, 3, 7)
    out["sparse-er+pendants"] = gbc.add_pendants(gbc.gen_er(600, 1.5, seed=5), 100, 3, 9)
    out["grid-holes"] = gbc.gen_grid(20, 20, 0.3, seed=2, largest_only=False)
    out["ba-tree"] = gbc.gen_ba(500, 1, 3)
    return out


def test_reduction_rules_match_host_and_networkx(gbc, datasets):
    nx = pytest.importorskip("networkx")
    rng = np.random.default_rng(0)
    for name, csr in _graphs(gbc, datasets).items():
        alive, _, folded = _fold_rounds(csr.row, csr.col, csr.n, csr.start, rng)
        info = gbc.Reduced(csr, on_host=True).info()
        assert folded == info["d1_folded"], name
        core_v = [v for v in range(csr.n) if alive[v]]
        blocks, aps = _blocks(csr.row, csr.col, core_v, alive)
        g = nx.Graph()
        g.add_nodes_from(core_v)
        keep = set(core_v)
        for v in core_v:
            g.add_edges_from((v, int(w)) for w in csr.col[csr.row[v]:csr.row[v + 1]] if int(w) in keep)
        ref = [tuple(sorted(c)) for c in nx.biconnected_components(g)] + [(v,) for v in core_v if g.degree(v) == 0]
        assert blocks == sorted(ref), name
        assert aps == set(nx.articulation_points(g)), name
        assert (len(blocks), len(aps)) == (info["blocks"], info["articulation_points"]), name

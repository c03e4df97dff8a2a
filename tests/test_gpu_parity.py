"""GPU parity: the CUDA engines (through the C ABI) against the CPU oracle.

Bars: distances, exact uint64 path counts and closeness sums bit-exact;
betweenness within 1e-9 relative (FP64 delta) or 1e-6 relative (FP32 delta)
of the FP64 oracle, measured as max |a-b| / max(|b|, 1) over vertices.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-9
TOL_F32 = 1e-6


def relerr(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if len(b) else 0.0


def to_orc(orc, csr):
    return orc.Graph(csr.row, csr.col, csr.start)


@pytest.fixture(scope="module")
def graphs(gpu, datasets):
    g = {}
    g["ba4096"] = gpu.gen_ba(4096, 4, 1)
    g["rmat12"] = gpu.gen_rmat(12, 8, seed=2)
    g["grid24"] = gpu.gen_grid(24, 24, 0.05, seed=3)
    g["er2k"] = gpu.gen_er(2000, 3.0, seed=4)          # disconnected
    g["karate"] = gpu.read_edgelist(datasets["karate.txt"])
    g["ia-fb"] = gpu.read_edgelist(datasets["ia-fb-messages.mtx"])
    g["rmat14"] = gpu.gen_rmat(14, 16, seed=2)           # 15 vertices above the hub degree
    # a star of 3000 leaves (a hub) joined to a 24x24 grid, plus isolated vertices
    grid = gpu.gen_grid(24, 24, 0.0, seed=1)
    n0 = grid.n
    rows, cols = [], []
    adj = [list(grid.col[grid.row[v]:grid.row[v + 1]]) for v in range(n0)]
    hub = n0
    adj.append([0] + list(range(n0 + 1, n0 + 3001)))
    adj[0].append(hub)
    for leaf in range(n0 + 1, n0 + 3001):
        adj.append([hub])
    adj += [[] for _ in range(5)]
    row = np.zeros(len(adj) + 1, np.int64)
    for v, a in enumerate(adj):
        row[v + 1] = row[v] + len(a)
    g["star+grid"] = gpu.CSR(row, np.array([x for a in adj for x in sorted(a)], np.int32))
    return g


def sources_of(csr, cap, seed=5):
    if csr.n - csr.start <= cap:
        return np.arange(csr.start, csr.n, dtype=np.int32)
    return np.random.default_rng(seed).choice(np.arange(csr.start, csr.n), cap, replace=False).astype(np.int32)


@pytest.mark.parametrize("name", ["ba4096", "rmat12", "grid24", "er2k", "karate", "rmat14", "star+grid"])
@pytest.mark.parametrize("lanes", [32, 128])
def test_sssp_bit_exact(gpu, orc, graphs, name, lanes):
    csr = graphs[name]
    og = to_orc(orc, csr)
    rng = np.random.default_rng(7)
    src = rng.integers(csr.start, csr.n, size=min(70, csr.n - csr.start)).astype(np.int32)
    with gpu.Graph(csr) as G:
        dist, sig, ovf = G.sssp(src, lanes=lanes)
    for i, s in enumerate(src):
        d0, s0, o0, _ = orc.sssp(og, int(s))
        assert np.array_equal(dist[i], d0), f"dist mismatch for source {s}"
        assert bool(ovf[i]) == bool(o0.any())
        if not o0.any():
            assert np.array_equal(sig[i], s0), f"sigma mismatch for source {s}"


@pytest.mark.parametrize("name", ["ba4096", "rmat12", "er2k", "karate", "ia-fb", "rmat14", "star+grid"])
def test_cc_bit_exact(gpu, orc, graphs, name):
    csr = graphs[name]
    og = to_orc(orc, csr)
    src = sources_of(csr, 3000)
    ref = orc.cc(og, src, nthreads=4)
    with gpu.Graph(csr) as G:
        got = G.cc(src)
        assert np.array_equal(got, ref)
        got_plain = G.cc(src[:50], engine=gpu.ENGINE_PLAIN)
        assert np.array_equal(got_plain, ref[:50])


@pytest.mark.parametrize("name", ["ba4096", "rmat12", "er2k", "karate", "rmat14", "star+grid", "grid24"])
def test_cc_direction_switching(gpu, orc, graphs, name):
    """Closeness on 128-lane groups with bottom-up levels on the large
    frontiers equals the oracle and the top-down-only run bit for bit, also
    on graphs with many components (lanes whose source lies elsewhere are
    masked out of the early exit)."""
    csr = graphs[name]
    src = sources_of(csr, 512)
    with gpu.Graph(csr) as G:
        a = G.cc(src, lanes=256, group_lanes=128)
        st = G.stats()
        b = G.cc(src, lanes=256, group_lanes=128, direction=1)
        stb = G.stats()
    ref = orc.cc(to_orc(orc, csr), src, nthreads=8)
    assert np.array_equal(a, ref) and np.array_equal(b, ref)
    assert stb["bottom_up_levels"] == 0
    if name in ("ba4096", "rmat12", "rmat14"):
        assert st["bottom_up_levels"] > 0


@pytest.mark.parametrize("side,width", [(6, 2), (14, 4), (30, 8)])
def test_path_count_widths(gpu, orc, side, width):
    """128-lane groups store exact path counts in 2 bytes and widen a batch to
    4 and then 8 bytes when a count does not fit; results stay bit-exact.
    Full grids from a corner: the largest count is C(2(side-1), side-1) -- 252,
    10.4M and 3.0e16 for sides 6, 14, 30.  A later call on the same graph starts
    at the width found (no redo)."""
    csr = gpu.gen_grid(side, side, 0.0, seed=1)
    og = orc.Graph(csr.row, csr.col)
    src = np.arange(0, min(csr.n, 128), dtype=np.int32)     # vertex 0 is a corner
    ref, novf = orc.bc(og, src, nthreads=8)
    assert novf == 0
    with gpu.Graph(csr) as G:
        got = G.bc(src, lanes=128, group_lanes=128, sigma_mode=gpu.SIGMA_EXACT)
        st = G.stats()
        assert st["sigma_bytes"] == width and st["group_lanes"] == 128
        assert relerr(got, ref) < TOL_F64
        launches = st["kernel_launches"]
        again = G.bc(src, lanes=128, group_lanes=128, sigma_mode=gpu.SIGMA_EXACT)
        assert G.stats()["sigma_bytes"] == width
        assert G.stats()["kernel_launches"] <= launches
        assert relerr(again, ref) < TOL_F64
        dist, sig, ovf = G.sssp(src[:4], lanes=128, group_lanes=128)
    for i in range(4):
        d0, s0, o0, _ = orc.sssp(og, int(src[i]))
        assert np.array_equal(dist[i], d0) and np.array_equal(sig[i], s0) and not ovf[i]
    d0, s0, _, _ = orc.sssp(og, 0)
    assert (int(s0.max()) > 0xFFFF) == (width > 2) and (int(s0.max()) > 0xFFFFFFFF) == (width > 4)


@pytest.mark.parametrize("name", ["rmat14", "grid24", "star+grid", "er2k"])
@pytest.mark.parametrize("threads", [128, 512])
def test_cta_shapes(gpu, orc, graphs, name, threads):
    """The level kernels of every CTA shape (128 / 512 threads against the
    default 256) give the oracle's betweenness and closeness, on 32- and
    128-lane groups, and closeness is the same for every direction-switch
    share (bu_share) and for top-down only."""
    csr = graphs[name]
    og = to_orc(orc, csr)
    src = sources_of(csr, 300)
    ref, _ = orc.bc(og, src, scaled=(name == "grid24"), nthreads=8)
    ref_cc = orc.cc(og, src, nthreads=8)
    with gpu.Graph(csr) as G:
        for group in (32, 128):
            got = G.bc(src, lanes=256, group_lanes=group, block_threads=threads)
            assert relerr(got, ref) < TOL_F64, (group, threads)
            assert np.array_equal(G.cc(src, lanes=256, group_lanes=group, block_threads=threads), ref_cc)
        for share in (1, 4, 64, 4096):
            assert np.array_equal(G.cc(src, lanes=256, group_lanes=128, block_threads=threads, bu_share=share), ref_cc)


@pytest.mark.parametrize("name", ["ba4096", "rmat12", "er2k", "karate", "rmat14", "star+grid"])
@pytest.mark.parametrize("sem", [0, 1])
def test_bc_fp64(gpu, orc, graphs, name, sem):
    csr = graphs[name]
    og = to_orc(orc, csr)
    src = sources_of(csr, 1500)
    ref, novf = orc.bc(og, src, semantics=sem, nthreads=4)
    assert novf == 0
    with gpu.Graph(csr) as G:
        got = G.bc(src, semantics=sem, delta_precision=gpu.DELTA_F64, sigma_mode=gpu.SIGMA_EXACT)
        assert relerr(got, ref) < TOL_F64
        st = G.stats()
        assert st["sources"] == len(src) and st["sigma_mode_used"] == gpu.SIGMA_EXACT


@pytest.mark.parametrize("name", ["ba4096", "rmat12", "rmat14"])
def test_bc_fp32_delta(gpu, orc, graphs, name):
    csr = graphs[name]
    og = to_orc(orc, csr)
    src = sources_of(csr, 1500)
    ref, _ = orc.bc(og, src, nthreads=4)
    with gpu.Graph(csr) as G:
        got = G.bc(src, delta_precision=gpu.DELTA_F32)
    assert relerr(got, ref) < TOL_F32


def test_bc_plain_engine(gpu, orc, graphs):
    csr = graphs["rmat12"]
    og = to_orc(orc, csr)
    src = np.arange(0, 64, dtype=np.int32)
    ref, _ = orc.bc(og, src)
    with gpu.Graph(csr) as G:
        got = G.bc(src, engine=gpu.ENGINE_PLAIN)
    assert relerr(got, ref) < TOL_F64


def test_bc_sampled_sources_and_duplicates(gpu, orc, graphs):
    csr = graphs["ba4096"]
    og = to_orc(orc, csr)
    rng = np.random.default_rng(3)
    src = rng.integers(0, csr.n, size=300).astype(np.int32)   # with repeats
    ref, _ = orc.bc(og, src, semantics=1)
    with gpu.Graph(csr) as G:
        got = G.bc(src, semantics=1, lanes=64)
    assert relerr(got, ref) < TOL_F64


def test_bc_reference_golden_karate(gpu, graphs):
    gold = np.loadtxt(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                                  "karate_BC_Score.txt"), skiprows=1)
    csr = graphs["karate"]
    with gpu.Graph(csr) as G:
        got = G.bc(np.arange(1, csr.n, dtype=np.int32), semantics=gpu.BC_REFERENCE)
    # the golden file holds FP32 values printed with %f
    assert np.max(np.abs(got[1:] - gold) / np.maximum(gold, 1.0)) < 2e-6


def test_sigma_overflow_log_mode(gpu, orc):
    # a full 80x80 grid: corner-to-corner path counts ~C(158,79) > 2^64
    csr = gpu.gen_grid(80, 80, 0.0, seed=1)
    og = to_orc(orc, csr)
    src = np.array([0, 79, 3200, 6399], dtype=np.int32)
    ref, novf = orc.bc(og, src, scaled=True)
    assert novf > 0
    with gpu.Graph(csr) as G:
        with pytest.raises(gpu.GbcError):
            G.bc(src, sigma_mode=gpu.SIGMA_EXACT)
        got = G.bc(src)   # AUTO: exact, then wide form for overflowing batches
        st = G.stats()
        assert st["sigma_mode_used"] == gpu.SIGMA_WIDE
        assert relerr(got, ref) < TOL_F64
        dist, sig, ovf = G.sssp(src)
        assert ovf.all()


@pytest.mark.parametrize("sparse,light", [(0, 0), (32, 0), (2, 0), (2, 1 << 20), (-1, -1)])
def test_expansion_modes_agree(gpu, orc, graphs, sparse, light):
    """Lane-parallel only (sparse=0), edge-parallel only (sparse=32), no
    one-thread tasks (light=0), one-thread tasks for every non-hub entry and
    the defaults all give the same exact results, also after switching modes
    on one engine."""
    csr = graphs["star+grid"]
    og = to_orc(orc, csr)
    src = sources_of(csr, 400, seed=9)
    ref, _ = orc.bc(og, src, semantics=1)
    refcc = orc.cc(og, src)
    with gpu.Graph(csr) as G:
        G.bc(src[:64], semantics=1, lanes=96)   # capture with the defaults first
        got = G.bc(src, semantics=1, sparse_lanes=sparse, light_steps=light, lanes=96)
        assert relerr(got, ref) < TOL_F64
        assert np.array_equal(G.cc(src, sparse_lanes=sparse, light_steps=light, lanes=96), refcc)
        dist, sig, _ = G.sssp(src[:32], light_steps=light, sparse_lanes=sparse)
        for i, s in enumerate(src[:32]):
            rd, rs, _, _ = orc.sssp(og, int(s))
            assert np.array_equal(dist[i], rd) and np.array_equal(sig[i], rs)


def test_deep_graph_switches_level_width(gpu, orc):
    """A 700-vertex path is deeper than 8-bit levels allow: the engine
    switches to 16-bit levels and stays exact."""
    n = 700
    row = np.concatenate([[0], np.cumsum([1] + [2] * (n - 2) + [1])]).astype(np.int64)
    col = []
    for v in range(n):
        col += ([v - 1] if v > 0 else []) + ([v + 1] if v < n - 1 else [])
    csr = gpu.CSR(row, np.array(col, np.int32))
    og = to_orc(orc, csr)
    src = np.array([0, 5, 350, 699], np.int32)
    ref, _ = orc.bc(og, src)
    with gpu.Graph(csr) as G:
        assert relerr(G.bc(src), ref) < TOL_F64
        assert np.array_equal(G.cc(src), orc.cc(og, src))
        dist, _, _ = G.sssp(src)
        assert dist[0, 699] == 699


def test_edge_cases(gpu, orc):
    """A single vertex, isolated vertices, repeated sources, the all-sources
    call and a hub that is not vertex 0 (the device relabels by degree) all
    agree with the oracle."""
    one = gpu.CSR(np.zeros(2, np.int64), np.zeros(0, np.int32))
    with gpu.Graph(one) as G:
        assert np.array_equal(G.bc(), np.zeros(1)) and np.array_equal(G.cc(), np.zeros(1, np.int64))
        dist, sig, _ = G.sssp(np.array([0], np.int32))
        assert dist[0, 0] == 0 and sig[0, 0] == 1
    # path 0-1-2 plus isolated 3, and a star centred on the last vertex
    n = 12
    edges = [(0, 1), (1, 2)] + [(i, n - 1) for i in range(4, n - 1)]
    u = np.array([a for a, b in edges] + [b for a, b in edges], np.int32)
    v = np.array([b for a, b in edges] + [a for a, b in edges], np.int32)
    o = np.lexsort((v, u))
    row = np.concatenate([[0], np.cumsum(np.bincount(u, minlength=n))]).astype(np.int64)
    csr = gpu.CSR(row, v[o])
    og = to_orc(orc, csr)
    for src in (np.array([0, 0, 3, n - 1, n - 1, 5], np.int32), np.arange(n, dtype=np.int32)):
        ref, _ = orc.bc(og, src)
        refr, _ = orc.bc(og, src, semantics=1)
        with gpu.Graph(csr) as G:
            assert relerr(G.bc(src), ref) < TOL_F64
            assert relerr(G.bc(src, semantics=1, delta_precision=gpu.DELTA_F32), refr) < TOL_F32
            assert np.array_equal(G.cc(src), orc.cc(og, src))
            dist, sig, _ = G.sssp(src)
            for i, s in enumerate(src):
                d0, s0, _, _ = orc.sssp(og, int(s))
                assert np.array_equal(dist[i], d0) and np.array_equal(sig[i], s0)
    with gpu.Graph(csr) as G:
        ref, _ = orc.bc(og, np.arange(n))
        assert relerr(G.bc(), ref) < TOL_F64
        assert np.array_equal(G.cc(), orc.cc(og, np.arange(n)))


@pytest.mark.parametrize("name", ["ba4096", "rmat12", "grid24", "er2k", "karate", "rmat14", "star+grid"])
def test_group128_parity(gpu, orc, graphs, name):
    """128-lane groups (four lanes per thread): distances and path counts
    bit-exact, closeness exact, BC within tolerance in both semantics and
    both sweep precisions, also with the edge-parallel mode forced."""
    csr = graphs[name]
    og = to_orc(orc, csr)
    src = sources_of(csr, 300, seed=21)
    ref0, _ = orc.bc(og, src, semantics=0)
    ref1, _ = orc.bc(og, src, semantics=1)
    with gpu.Graph(csr) as G:
        for lanes in (128, 256):
            assert relerr(G.bc(src, group_lanes=128, lanes=lanes), ref0) < TOL_F64
            assert relerr(G.bc(src, group_lanes=128, lanes=lanes, semantics=1), ref1) < TOL_F64
            assert relerr(G.bc(src, group_lanes=128, lanes=lanes, delta_precision=gpu.DELTA_F32), ref0) < TOL_F32
        assert relerr(G.bc(src, group_lanes=128, lanes=128, sparse_lanes=128), ref0) < TOL_F64
        assert np.array_equal(G.cc(src, group_lanes=128, lanes=256), orc.cc(og, src))
        assert np.array_equal(G.cc(src, group_lanes=128, lanes=128, sparse_lanes=0), orc.cc(og, src))
        dist, sig, ovf = G.sssp(src[:130], group_lanes=128)
        for i, s in enumerate(src[:130]):
            d0, s0, o0, _ = orc.sssp(og, int(s))
            assert np.array_equal(dist[i], d0)
            if not o0.any():
                assert np.array_equal(sig[i], s0)


def test_group128_deep_and_wide(gpu, orc):
    """128-lane groups on a graph deeper than 8-bit levels and on a grid whose
    path counts overflow uint64 (wide form)."""
    n = 700
    row = np.concatenate([[0], np.cumsum([1] + [2] * (n - 2) + [1])]).astype(np.int64)
    col = []
    for v in range(n):
        col += ([v - 1] if v > 0 else []) + ([v + 1] if v < n - 1 else [])
    path = gpu.CSR(row, np.array(col, np.int32))
    og = to_orc(orc, path)
    src = np.array([0, 5, 350, 699], np.int32)
    with gpu.Graph(path) as G:
        assert relerr(G.bc(src, group_lanes=128), orc.bc(og, src)[0]) < TOL_F64
        assert np.array_equal(G.cc(src, group_lanes=128), orc.cc(og, src))
    grid = gpu.gen_grid(80, 80, 0.0, seed=1)
    og = to_orc(orc, grid)
    src = np.array([0, 79, 3200, 6399], dtype=np.int32)
    ref, novf = orc.bc(og, src, scaled=True)
    assert novf > 0
    with gpu.Graph(grid) as G:
        got = G.bc(src, group_lanes=128)
        assert G.stats()["sigma_mode_used"] == gpu.SIGMA_WIDE
        assert relerr(got, ref) < TOL_F64


@pytest.mark.parametrize("name", ["grid24", "er2k", "ba4096", "rmat12", "karate", "star+grid"])
def test_one_lane_per_task(gpu, orc, graphs, name):
    """One lane per task (group_lanes = 1: lane-major state, (vertex, lane)
    entries, discovery by compare-and-swap on the level) gives the oracle's
    betweenness in both semantics and both delta precisions, exact closeness,
    distances and path counts -- also on graphs with many components and with
    a 3000-leaf hub, which this mode expands one thread per entry."""
    csr = graphs[name]
    og = to_orc(orc, csr)
    src = sources_of(csr, 200)
    with gpu.Graph(csr) as G:
        for sem in (0, 1):
            ref, novf = orc.bc(og, src, semantics=sem, nthreads=8)
            assert novf == 0
            got = G.bc(src, semantics=sem, group_lanes=1, sigma_mode=gpu.SIGMA_EXACT)
            st = G.stats()
            assert st["group_lanes"] == 1 and st["lanes"] >= 32
            assert relerr(got, ref) < TOL_F64
            got32 = G.bc(src, semantics=sem, group_lanes=1, delta_precision=gpu.DELTA_F32)
            assert relerr(got32, ref) < TOL_F32
        assert np.array_equal(G.cc(src, group_lanes=1), orc.cc(og, src, nthreads=8))
        dist, sig, ovf = G.sssp(src[:6], group_lanes=1)
    for i in range(6):
        d0, s0, o0, _ = orc.sssp(og, int(src[i]))
        assert np.array_equal(dist[i], d0) and not ovf[i] and np.array_equal(sig[i], s0)


def test_one_lane_per_task_wide_and_partial_batch(gpu, orc):
    """One lane per task on a grid whose path counts overflow uint64 (wide
    form), and with a batch narrower than the engine (unused lanes)."""
    grid = gpu.gen_grid(80, 80, 0.0, seed=1)
    og = to_orc(orc, grid)
    src = np.array([0, 79, 3200, 6399, 17, 4100], dtype=np.int32)
    ref, novf = orc.bc(og, src, scaled=True)
    assert novf > 0
    with gpu.Graph(grid) as G:
        got = G.bc(src, group_lanes=1, lanes=64)
        st = G.stats()
        assert st["sigma_mode_used"] == gpu.SIGMA_WIDE and st["group_lanes"] == 1
        assert relerr(got, ref) < TOL_F64
        assert np.array_equal(G.cc(src, group_lanes=1, lanes=64), orc.cc(og, src))


def test_group128_grid_queue_growth(gpu, orc):
    """128-lane groups of random sources on a grid: a (vertex, group) task
    recurs at up to 128 levels, far beyond the first frontier queue, which
    has to grow several times within one batch.  Betweenness (wide path
    counts) and closeness against the oracle."""
    grid = gpu.gen_grid(200, 200, 0.05, seed=3)
    og = to_orc(orc, grid)
    src = np.random.default_rng(7).choice(grid.n, 512, replace=False).astype(np.int32)
    ref, _ = orc.bc(og, src, scaled=True, nthreads=8)
    with gpu.Graph(grid) as G:
        got = G.bc(src, lanes=512, group_lanes=128)
        st = G.stats()
        cc = G.cc(src, lanes=512, group_lanes=128)
    assert st["group_lanes"] == 128 and st["sigma_mode_used"] == gpu.SIGMA_WIDE
    assert st["frontier_entries"] > 8 * 4 * grid.n    # beyond the initial queue of 8 entries per (vertex, group)
    assert relerr(got, ref) < TOL_F64
    assert np.array_equal(cc, orc.cc(og, src, nthreads=8))


def test_group128_hub_with_wide_sigma(gpu, orc):
    """A hub (1280 neighbours, above the CTA-wide threshold) whose path counts
    overflow uint64: an 80x80 grid with the hub joined to the 39 vertices of
    the anti-diagonal i+j=120 (path counts up to ~1e35 from the corner) and
    to 1241 leaves.  The hub's sigma and delta are merged across the CTA's
    warps in the wide form; BC against the oracle's scaled FP64 Brandes."""
    side = 80
    grid = gpu.gen_grid(side, side, 0.0, seed=1)
    n0 = grid.n
    adj = [list(grid.col[grid.row[v]:grid.row[v + 1]]) for v in range(n0)]
    hub = n0
    diag = [i * side + (120 - i) for i in range(120 - (side - 1), side)]
    leaves = list(range(n0 + 1, n0 + 1 + 1280 - len(diag)))
    adj.append(sorted(diag + leaves))
    for v in diag:
        adj[v].append(hub)
    for v in leaves:
        adj.append([hub])
    row = np.concatenate([[0], np.cumsum([len(a) for a in adj])]).astype(np.int64)
    col = np.concatenate([np.sort(np.array(a, np.int32)) for a in adj]).astype(np.int32)
    csr = gpu.CSR(row, col)
    assert row[hub + 1] - row[hub] == 1280
    og = to_orc(orc, csr)
    src = np.array([0, 1, side, side + 1, 79, 6399, leaves[0]], np.int32)
    ref, novf = orc.bc(og, src, scaled=True)
    assert novf > 0
    with gpu.Graph(csr) as G:
        for dp in (gpu.DELTA_F64, gpu.DELTA_F32):
            got = G.bc(src, group_lanes=128, delta_precision=dp)
            assert G.stats()["sigma_mode_used"] == gpu.SIGMA_WIDE
            assert relerr(got, ref) < (TOL_F64 if dp == gpu.DELTA_F64 else TOL_F32)
        assert np.array_equal(G.cc(src, group_lanes=128), orc.cc(og, src))


def king_graph(gpu, side, drop, seed):
    """A side x side grid with diagonals (degree up to 8), a fraction of the edges dropped."""
    r, c = np.divmod(np.arange(side * side), side)
    u, v = [], []
    for dr, dc in ((0, 1), (1, -1), (1, 0), (1, 1)):
        ok = (r + dr < side) & (c + dc >= 0) & (c + dc < side)
        u.append(np.nonzero(ok)[0])
        v.append(np.nonzero(ok)[0] + dr * side + dc)
    u, v = np.concatenate(u), np.concatenate(v)
    keep = np.random.default_rng(seed).random(len(u)) >= drop
    u, v = u[keep], v[keep]
    a, b = np.concatenate([u, v]), np.concatenate([v, u])
    o = np.lexsort((b, a))
    row = np.zeros(side * side + 1, np.int64)
    np.add.at(row, a + 1, 1)
    return gpu.CSR(np.cumsum(row), b[o].astype(np.int32))


@pytest.mark.parametrize("kind", ["grid", "king"])
def test_one_lane_neighbour_table(gpu, orc, kind):
    """Deep graphs of degree <= 4 and <= 8 run one lane per task by default and
    read neighbours from the padded table (one or two 16-byte slots per vertex):
    betweenness in both semantics, closeness, distances and path counts against
    the oracle (level-scaled where path counts pass 2^64)."""
    csr = gpu.gen_grid(70, 70, 0.05, seed=9) if kind == "grid" else king_graph(gpu, 64, 0.3, 2)
    deg = np.diff(csr.row)
    assert deg.max() <= (4 if kind == "grid" else 8) and (kind == "grid" or deg.max() > 4)
    og = to_orc(orc, csr)
    src = sources_of(csr, 150)
    with gpu.Graph(csr) as G:
        for sem in (0, 1):
            ref, _ = orc.bc(og, src, semantics=sem, scaled=True, nthreads=8)
            got = G.bc(src, semantics=sem)
            assert G.stats()["group_lanes"] == 1
            assert relerr(got, ref) < TOL_F64
        assert np.array_equal(G.cc(src), orc.cc(og, src, nthreads=8))
        dist, sig, ovf = G.sssp(src[:4])
    for i in range(4):
        d0, s0, o0, _ = orc.sssp(og, int(src[i]))
        assert np.array_equal(dist[i], d0)
        if not ovf[i] and not o0.any():
            assert np.array_equal(sig[i], s0)

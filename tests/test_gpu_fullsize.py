"""GPU parity at the full sizes of the benchmark configurations.

  * R-MAT scale 22, edge factor 16 (a=.57, b=.19, c=.19; 4.2M vertices,
    128M directed entries), the sampled-betweenness workload of bench.py;
  * the 1024 x 1024 grid with 5% of its edges removed (seed 3), largest
    component only: 2000+ BFS levels, path counts far beyond uint64 and FP64.

Checks, through the C ABI:
  * per-vertex betweenness of a few sampled sources against the FP64 oracle
    (its level-normalised form on the grid): within 1e-9 relative with FP64
    delta, 1e-6 with FP32 delta;
  * closeness sums of those sources bit-exact, distances and exact path
    counts bit-exact where they fit in uint64;
  * a size-independent identity over a whole 1024-source batch: every
    shortest s-t path has d(s,t) - 1 interior vertices, so with Brandes
    semantics sum_v BC(v) = sum_s (CC(s) - (|comp(s)| - 1)) exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-9
TOL_F32 = 1e-6
# FP32 delta rounds delta and rho once per level; over the grid's 2000+ levels
# the relative error compounds (measured 1.05e-6 on 16 sources), so the deep
# grid gets its own bound.  R-MAT's handful of levels stays within TOL_F32.
TOL_F32_DEEP = 1e-5


def relerr(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.fixture(scope="module")
def rmat22(gpu):
    csr = gpu.gen_rmat(22, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    deg = np.diff(csr.row)
    cand = np.nonzero(deg > 0)[0].astype(np.int32)
    sample = np.random.default_rng(4).choice(cand, 16384, replace=False).astype(np.int32)
    return csr, sample


@pytest.fixture(scope="module")
def grid1024(gpu):
    return gpu.gen_grid(1024, 1024, 0.05, seed=3, largest_only=True)


def component_sizes(csr):
    cs = pytest.importorskip("scipy.sparse.csgraph")
    sp = pytest.importorskip("scipy.sparse")
    a = sp.csr_matrix((np.ones(len(csr.col), np.int8), csr.col, csr.row), shape=(csr.n, csr.n))
    _, lab = cs.connected_components(a, directed=False)
    return np.bincount(lab)[lab]


def test_rmat22_sampled_sources_vs_oracle(gpu, orc, rmat22):
    csr, sample = rmat22
    assert csr.n == 1 << 22 and csr.m == 128_311_672
    src = sample[:8]
    og = orc.Graph(csr.row, csr.col)
    ref, _ = orc.bc(og, src, semantics=orc.BC_BRANDES, nthreads=16)
    with gpu.Graph(csr) as G:
        b64 = G.bc(src, delta_precision=gpu.DELTA_F64)
        b32 = G.bc(src, delta_precision=gpu.DELTA_F32)
        cc = G.cc(src)
        dist, sig, ovf = G.sssp(src[:2])
    assert relerr(b64, ref) < TOL_F64
    assert relerr(b32, ref) < TOL_F32
    assert np.array_equal(cc, orc.cc(og, src, nthreads=16))
    for i, s in enumerate(src[:2]):
        d, sg, so, _ = orc.sssp(og, int(s))
        assert np.array_equal(dist[i], d)
        fits = ~so
        assert np.array_equal(sig[i][fits], sg[fits])


def test_rmat22_batch_identity(gpu, rmat22):
    csr, sample = rmat22
    src = sample[:1024]
    comp = component_sizes(csr)
    with gpu.Graph(csr) as G:
        bc = G.bc(src, delta_precision=gpu.DELTA_F64)
        cc = G.cc(src)
    interior = int(cc.sum()) - int((comp[src] - 1).sum())
    assert abs(float(bc.sum()) - interior) / interior < TOL_F64


def test_grid1024_sampled_sources_vs_oracle(gpu, orc, grid1024):
    csr = grid1024
    assert 990_000 < csr.n < 1 << 20
    src = np.random.default_rng(8).choice(csr.n, 16, replace=False).astype(np.int32)
    og = orc.Graph(csr.row, csr.col)
    ref, _ = orc.bc(og, src, semantics=orc.BC_BRANDES, scaled=True, nthreads=16)
    with gpu.Graph(csr) as G:
        b64 = G.bc(src, delta_precision=gpu.DELTA_F64)
        st = G.stats()
        b32 = G.bc(src, delta_precision=gpu.DELTA_F32)
        cc = G.cc(src)
    assert st["sigma_mode_used"] == gpu.SIGMA_WIDE   # corner-to-corner counts pass 2^64 at ~34 hops
    assert relerr(b64, ref) < TOL_F64
    assert relerr(b32, ref) < TOL_F32_DEEP
    assert np.array_equal(cc, orc.cc(og, src, nthreads=16))
    # the identity on the same sources (one component)
    interior = int(cc.sum()) - len(src) * (csr.n - 1)
    assert abs(float(b64.sum()) - interior) / interior < TOL_F64


def test_c1_ba4096_all_sources(gpu, orc):
    """The plain exact configuration whole: BA n=4096, m=4, seed 1, every
    vertex a source, betweenness with FP64 delta in both semantics and
    closeness, against the FP64 oracle (about 1.5 s of oracle time)."""
    csr = gpu.gen_ba(4096, 4, 1)
    og = orc.Graph(csr.row, csr.col)
    src = np.arange(csr.n, dtype=np.int32)
    with gpu.Graph(csr) as G:
        for sem in (orc.BC_BRANDES, orc.BC_REFERENCE):
            ref, novf = orc.bc(og, src, semantics=sem, nthreads=16)
            assert novf == 0
            got = G.bc(None, semantics=sem, delta_precision=gpu.DELTA_F64, sigma_mode=gpu.SIGMA_EXACT)
            assert relerr(got, ref) < TOL_F64, sem
            assert G.stats()["sources"] == csr.n
        cc = G.cc(None)
    assert np.array_equal(cc, orc.cc(og, src, nthreads=16))


def test_grid1024_256_of_8192_sources_vs_oracle(gpu, orc, grid1024):
    """The deep configuration on 256 of its 8,192 uniformly sampled sources
    (seed 3, as the bench draws them), on 32-lane groups and one lane per task:
    betweenness in wide form against the oracle's level-normalised FP64 form,
    closeness bit-exact."""
    csr = grid1024
    sample = np.random.default_rng(3).choice(csr.n, 8192, replace=False).astype(np.int32)
    src = sample[:256]
    og = orc.Graph(csr.row, csr.col)
    ref, _ = orc.bc(og, src, semantics=orc.BC_BRANDES, scaled=True, nthreads=16)
    ref_cc = orc.cc(og, src, nthreads=16)
    with gpu.Graph(csr) as G:
        # 32-lane groups, and one lane per task (what the autotuner picks on this graph)
        for group in (32, 1):
            b64 = G.bc(src, delta_precision=gpu.DELTA_F64, group_lanes=group)
            assert G.stats()["group_lanes"] == group
            b32 = G.bc(src, delta_precision=gpu.DELTA_F32, group_lanes=group)
            cc = G.cc(src, group_lanes=group)
            assert relerr(b64, ref) < TOL_F64, group
            assert relerr(b32, ref) < TOL_F32_DEEP, group
            assert np.array_equal(cc, ref_cc), group

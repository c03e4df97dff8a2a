"""GPU: the D1 + block reduction end to end, the struct-CSR drop-in entry
points, and the device-pointer entry points, against the oracle and the
reference's own outputs (golden fixtures)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from compat_structs import bind, build_dropin_driver, load

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
STRUCT = json.load(open(os.path.join(GOLDEN, "structure.json")))


def fixture(name):
    return np.load(os.path.join(GOLDEN, name.split(".")[0] + ".npz"))


@pytest.mark.parametrize("name", sorted(STRUCT))
def test_reduced_cc_matches_reference(gpu, datasets, name):
    csr = gpu.read_edgelist(datasets[name])
    R = gpu.Reduced(csr)
    got = R.cc()
    assert np.array_equal(got[csr.start:], fixture(name)["cc_ref"][csr.start:])
    info = R.info()
    st = STRUCT[name]
    assert (info["d1_folded"], info["articulation_points"]) == (st["d1"], st["ap"])


@pytest.mark.parametrize("case", ["rmat14+pendants", "sparse-er+pendants", "grid-holes"])
def test_reduced_cc_disconnected(gpu, orc, case):
    if case == "rmat14+pendants":
        csr = gpu.add_pendants(gpu.gen_rmat(14, 4, seed=5), 3000, 3, 9)
    elif case == "sparse-er+pendants":
        csr = gpu.add_pendants(gpu.gen_er(4000, 1.5, seed=5), 600, 3, 9)
    else:
        csr = gpu.gen_grid(40, 40, 0.3, seed=2, largest_only=False)
    og = orc.Graph(csr.row, csr.col)
    ref = orc.cc(og, np.arange(csr.n), nthreads=8)
    assert np.array_equal(gpu.Reduced(csr).cc(), ref)


def test_dropin_entry_points(gpu, datasets):
    L = bind(gpu.lib())
    for name in ["karate.txt", "dolphins.txt", "ia-fb-messages.mtx", "testdata2.txt"]:
        fx = fixture(name)
        g, c = load(L, datasets[name])
        vs = c.contents.csrVSize
        bcs = (C.c_float * vs)()
        L.computeBC(c, bcs)
        bc = np.frombuffer(bcs, np.float32).astype(np.float64)
        ref = fx["bc_ref_f32"].astype(np.float64)
        assert np.max(np.abs(bc[:-1] - ref) / np.maximum(np.abs(ref), 1.0)) < 5e-5, name
        shs = (C.c_float * vs)()
        L.computeBC_shareBased(c, shs)
        sh = np.frombuffer(shs, np.float32).astype(np.float64)
        ref = fx["bc_shared_ref_f32"].astype(np.float64)
        assert np.max(np.abs(sh[:-1] - ref) / np.maximum(np.abs(ref), 1.0)) < 5e-5, name
        ccs = (C.c_int * vs)()
        L.computeCC(c, ccs)
        cc = np.frombuffer(ccs, np.int32)[:-1]
        assert np.array_equal(cc[c.contents.startNodeID:], fx["cc_ref"][c.contents.startNodeID:].astype(np.int32))
        L.gpu_vb(c)
        assert np.array_equal(np.ctypeslib.as_array(c.contents.CCs, shape=(vs - 1,)), cc)
        L.gpu_fan(g, c)
        assert np.array_equal(np.ctypeslib.as_array(c.contents.CCs, shape=(vs - 1,)), cc)
        g2, c2 = load(L, datasets[name])
        out = (C.c_int * (2 * vs))()
        L.compute_D1_AP_CC_shareBased_DegreeOrder(c2, out)
        d1ap = np.frombuffer(out, np.int32)[:vs - 1]
        s = c2.contents.startNodeID
        assert np.array_equal(d1ap[s:], fx["d1ap_cc_ref"][s:].astype(np.int32)), name
        st = STRUCT[name]
        assert (c2.contents.foldedDegreeOneCount, c2.contents.ap_count) == (st["d1"], st["ap"])


@pytest.mark.parametrize("name", sorted(STRUCT))
def test_dropin_closeness_variants(gpu, datasets, name):
    """computeCC_shareBased (Seq_CC/CC.cpp:122), compute_D1_CC (CC.cpp:418)
    and preprocess_then_parallel_sharedBased_DegreeOrder
    (parallel_CC/para_CC.cu:61) through the struct-CSR drop-in on every
    shipped dataset, against the reference's own closeness outputs."""
    L = bind(gpu.lib())
    fx = fixture(name)
    g, c = load(L, datasets[name])
    vs, s = c.contents.csrVSize, c.contents.startNodeID
    out = (C.c_int * (2 * vs))()
    L.computeCC_shareBased(c, out)
    assert np.array_equal(np.frombuffer(out, np.int32)[s:vs - 1], fx["cc_ref"][s:].astype(np.int32))
    g, c = load(L, datasets[name])
    out = (C.c_int * (2 * vs))()
    L.compute_D1_CC(c, out)
    assert np.array_equal(np.frombuffer(out, np.int32)[s:vs - 1], fx["cc_ref"][s:].astype(np.int32))
    assert c.contents.foldedDegreeOneCount == STRUCT[name]["d1"]   # the struct is left folded, as the reference leaves it
    g, c = load(L, datasets[name])
    L.preprocess_then_parallel_sharedBased_DegreeOrder(c)
    got = np.ctypeslib.as_array(c.contents.CCs, shape=(vs - 1,))
    assert np.array_equal(got[s:], fx["d1ap_cc_ref"][s:].astype(np.int32))


def write_edgelist_1based(csr, path):
    """The reference's text format, 1-based ids (slot 0 stays phantom, so an
    isolated vertex 0 cannot flip the base detection)."""
    u = np.repeat(np.arange(csr.n), np.diff(csr.row))
    v = csr.col
    keep = u < v
    with open(path, "w") as f:
        f.write(f"{csr.n} {int(keep.sum())}\n")
        for a, b in zip(u[keep] + 1, v[keep] + 1):
            f.write(f"{a} {b}\n")


@pytest.mark.parametrize("case", ["er+pendants", "rmat+pendants", "counterexample"])
def test_dropin_d1_cc_disconnected(gpu, orc, tmp_path, case):
    """compute_D1_CC on disconnected graphs with pendant trees equals plain
    BFS closeness: the folded vertices are recovered with their own
    component's size (the reference's totalNodeNumber is wrong there)."""
    if case == "er+pendants":
        csr = gpu.add_pendants(gpu.gen_er(3000, 1.5, seed=7), 500, 3, 4)
    elif case == "rmat+pendants":
        csr = gpu.add_pendants(gpu.gen_rmat(12, 4, seed=3), 800, 3, 5)
    else:   # a triangle with a pendant vertex, and a separate triangle
        csr = gpu.CSR(np.array([0, 2, 4, 7, 8, 10, 12, 14]),
                      np.array([1, 2, 0, 2, 0, 1, 3, 2, 5, 6, 4, 6, 4, 5], np.int32))
    path = str(tmp_path / "g.txt")
    write_edgelist_1based(csr, path)
    L = bind(gpu.lib())
    g, c = load(L, path)
    vs = c.contents.csrVSize
    assert vs - 1 == csr.n + 1
    out = (C.c_int * (2 * vs))()
    L.compute_D1_CC(c, out)
    got = np.frombuffer(out, np.int32)[1:vs - 1].astype(np.int64)
    ref = orc.cc(orc.Graph(csr.row, csr.col), np.arange(csr.n), nthreads=8)
    assert np.array_equal(got, ref)
    assert c.contents.foldedDegreeOneCount > 0


def test_graph_vertex_weights(gpu, orc):
    """gbc_graph_set_weights: weighted closeness sums against the oracle's
    weighted form; reach-weighted betweenness of the folded graph, assembled
    with the folding's pair counts, against plain Brandes of the whole
    graph; weights cleared give the unweighted results back."""
    csr = gpu.add_pendants(gpu.gen_rmat(11, 6, seed=4), 300, 3, 6)
    rng = np.random.default_rng(2)
    w = rng.integers(0, 6, csr.n).astype(np.int32)
    ff = rng.integers(0, 1000, csr.n).astype(np.int64)
    og = orc.Graph(csr.row, csr.col)
    src = np.arange(0, csr.n, 3, dtype=np.int32)
    with gpu.Graph(csr) as G:
        G.set_weights(w, ff)
        got = G.cc(src)
        with pytest.raises(gpu.GbcError):
            G.cc(src[:4], engine=gpu.ENGINE_PLAIN)
        with pytest.raises(gpu.GbcError):
            G.bc(src[:4], semantics=gpu.BC_REFERENCE)
        G.set_weights(None, None)
        plain = G.cc(src)
    assert np.array_equal(got, orc.cc(og, src, w=w, ff=ff, nthreads=8))
    assert np.array_equal(plain, orc.cc(og, src, nthreads=8))
    R = gpu.Reduced(csr)
    core, cw, cv = R.core_graph()
    with gpu.Graph(core) as G:
        G.set_weights(cw)
        core_bc = G.bc(None, delta_precision=gpu.DELTA_F64)
    full = R.assemble_bc(core_bc)
    ref, _ = orc.bc(og, np.arange(csr.n), nthreads=8)
    assert float(np.max(np.abs(full - ref) / np.maximum(np.abs(ref), 1.0))) < 1e-9


@pytest.mark.parametrize("name", ["tech-WHOIS.mtx", "ca-HepPh.mtx", "caida.mtx", "ia-email-EU.mtx"])
def test_dropin_bc_vs_reference_large_datasets(gpu, datasets, name):
    """computeBC through the drop-in against the reference's own FP32 output on
    the larger shipped datasets; the reference's FP32 sums drift by up to
    ~1.2e-3 relative from exact values there (the oracle tests pin that)."""
    L = bind(gpu.lib())
    g, c = load(L, datasets[name])
    vs = c.contents.csrVSize
    bcs = (C.c_float * vs)()
    L.computeBC(c, bcs)
    s = c.contents.startNodeID
    bc = np.frombuffer(bcs, np.float32).astype(np.float64)[s:vs - 1]
    ref = fixture(name)["bc_ref_f32"].astype(np.float64)[s:]
    err = np.abs(bc - ref) / np.maximum(np.abs(ref), 1.0)
    assert err.max() < 2e-3 and np.quantile(err, 0.99) < 2e-4


def test_karate_golden_through_dropin(gpu, datasets):
    L = bind(gpu.lib())
    g, c = load(L, datasets["karate.txt"])
    vs = c.contents.csrVSize
    bcs = (C.c_float * vs)()
    L.computeBC(c, bcs)
    gold = np.loadtxt(os.path.join(GOLDEN, "karate_BC_Score.txt"), skiprows=1)
    got = np.frombuffer(bcs, np.float32)[1:vs - 1].astype(np.float64)
    assert np.max(np.abs(got - gold) / np.maximum(gold, 1.0)) < 2e-6


def test_device_pointer_entry_points(gpu, orc):
    torch = pytest.importorskip("torch")
    csr = gpu.gen_ba(3000, 3, 4)
    og = orc.Graph(csr.row, csr.col)
    src = np.arange(0, 3000, 3, dtype=np.int32)
    L = gpu.lib()
    d_row = torch.from_numpy(csr.row).cuda()
    d_col = torch.from_numpy(csr.col).cuda()
    h = C.c_void_p()
    gpu.check(L.gbc_graph_create_device(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), csr.n,
                                        csr.m, C.byref(h)))
    d_src = torch.from_numpy(src).cuda()
    d_bc = torch.empty(csr.n, dtype=torch.float64, device="cuda")
    d_cc = torch.empty(len(src), dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    o = gpu.options()
    gpu.check(L.gbc_bc_device(h, C.c_void_p(d_src.data_ptr()), len(src), C.byref(o), C.c_void_p(d_bc.data_ptr()),
                              C.c_void_p(st.cuda_stream)))
    gpu.check(L.gbc_cc_device(h, C.c_void_p(d_src.data_ptr()), len(src), C.byref(o), C.c_void_p(d_cc.data_ptr()),
                              C.c_void_p(st.cuda_stream)))
    torch.cuda.synchronize()
    ref, _ = orc.bc(og, src)
    assert np.max(np.abs(d_bc.cpu().numpy() - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-9
    assert np.array_equal(d_cc.cpu().numpy(), orc.cc(og, src))
    L.gbc_graph_destroy(h)


@pytest.mark.parametrize("case", ["karate", "ca-HepPh", "caida", "rmat13+pendants", "forest+er", "rmat13+cycles",
                                  "rmat13+cycles+pendants", "chain-of-blocks", "grid-holes"])
@pytest.mark.parametrize("host", [False, True])
def test_reduced_bc_matches_plain_brandes(gpu, orc, datasets, case, host):
    """Betweenness through D1 folding and the block split (reach-weighted
    Brandes inside every block with clone weights on the device, plus the
    pairs each articulation point separates and the folded pair counts)
    equals plain Brandes of the whole graph, on graphs with hundreds to
    thousands of articulation points, for both reductions."""
    if case == "karate":
        csr = gpu.read_edgelist(datasets["karate.txt"])
    elif case == "ca-HepPh":
        csr = gpu.read_edgelist(datasets["ca-HepPh.mtx"])
    elif case == "caida":
        csr = gpu.read_edgelist(datasets["caida.mtx"])
    elif case == "rmat13+pendants":
        csr = gpu.add_pendants(gpu.gen_rmat(13, 4, seed=5), 2500, 3, 9)
    elif case == "forest+er":
        csr = gpu.add_pendants(gpu.gen_er(3000, 1.2, seed=7), 800, 3, 11)
    elif case == "rmat13+cycles":
        csr = gpu.add_cycles(gpu.gen_rmat(13, 4, seed=5), 2000, 3, 6, 4)
    elif case == "rmat13+cycles+pendants":
        csr = gpu.add_pendants(gpu.add_cycles(gpu.gen_rmat(13, 4, seed=5), 1500, 3, 6, 4), 1500, 3, 9)
    elif case == "chain-of-blocks":
        csr = _chain_of_blocks(gpu)
    else:
        csr = gpu.gen_grid(60, 60, 0.3, seed=2, largest_only=False)
    og = orc.Graph(csr.row, csr.col, csr.start)
    ref, _ = orc.bc(og, np.arange(csr.start, csr.n), semantics=orc.BC_BRANDES, nthreads=8)
    R = gpu.Reduced(csr, on_host=host)
    info = R.info()
    if case in ("ca-HepPh", "rmat13+cycles", "rmat13+cycles+pendants", "chain-of-blocks"):
        assert info["articulation_points"] > 50, info
    for delta, tol in ((gpu.DELTA_F64, 1e-9), (gpu.DELTA_F32, 1e-6)):
        got = R.bc(delta_precision=delta)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) < tol, (case, delta)
    with pytest.raises(gpu.GbcError):
        R.bc(semantics=gpu.BC_REFERENCE)


def _csr_from_edges(gpu, edges, n):
    e = np.asarray(edges, np.int64).reshape(-1, 2)
    u = np.concatenate([e[:, 0], e[:, 1]])
    v = np.concatenate([e[:, 1], e[:, 0]])
    o = np.lexsort((v, u))
    u, v = u[o], v[o]
    row = np.zeros(n + 1, np.int64)
    np.add.at(row, u + 1, 1)
    return gpu.CSR(np.cumsum(row), v.astype(np.int32))


def _chain_of_blocks(gpu):
    """Cycles of 3 to 7 vertices chained by shared vertices and bridges, with
    pendant paths and a separate triangle: many articulation points."""
    rng = np.random.default_rng(9)
    edges, nxt, join = [], 1, 0
    for k in range(60):
        size = int(rng.integers(3, 8))
        cyc = [join] + list(range(nxt, nxt + size - 1))
        nxt += size - 1
        edges += [(cyc[i], cyc[(i + 1) % size]) for i in range(size)]
        join = cyc[int(rng.integers(0, size))]
        if k % 7 == 3:                       # a bridge to the next cycle
            edges.append((join, nxt))
            join, nxt = nxt, nxt + 1
        if k % 5 == 1:                       # a pendant path
            edges += [(cyc[1], nxt), (nxt, nxt + 1)]
            nxt += 2
    edges += [(nxt, nxt + 1), (nxt + 1, nxt + 2), (nxt + 2, nxt)]
    return _csr_from_edges(gpu, edges, nxt + 4)   # and one isolated vertex


@pytest.mark.parametrize("case", ["karate", "ca-HepPh", "caida", "tech-WHOIS", "ia-email-EU", "testdata1",
                                  "chain-of-blocks", "rmat14+pendants", "er+pendants", "grid-holes", "ba-tree",
                                  "path-701", "star-2000"])
def test_device_reduction_equals_host(gpu, datasets, case):
    """gbc_reduce (folding rounds + Tarjan-Vishkin blocks on the device) and
    gbc_reduce_host (sequential folding + DFS) give the same folded vertices,
    articulation points, blocks, block graph and clone weights, and the same
    closeness (exact) and betweenness."""
    named = {"karate": "karate.txt", "ca-HepPh": "ca-HepPh.mtx", "caida": "caida.mtx", "tech-WHOIS": "tech-WHOIS.mtx",
             "ia-email-EU": "ia-email-EU.mtx", "testdata1": "testdata1.txt"}
    if case in named:
        csr = gpu.read_edgelist(datasets[named[case]])
    elif case == "chain-of-blocks":
        csr = _chain_of_blocks(gpu)
    elif case == "rmat14+pendants":
        csr = gpu.add_pendants(gpu.gen_rmat(14, 4, seed=5), 3000, 3, 9)
    elif case == "er+pendants":
        csr = gpu.add_pendants(gpu.gen_er(4000, 1.5, seed=5), 600, 3, 9)
    elif case == "grid-holes":
        csr = gpu.gen_grid(60, 60, 0.3, seed=2, largest_only=False)
    elif case == "ba-tree":
        csr = gpu.gen_ba(3000, 1, 3)
    elif case == "path-701":
        csr = _csr_from_edges(gpu, [(i, i + 1) for i in range(700)], 701)
    else:
        csr = _csr_from_edges(gpu, [(0, i) for i in range(1, 2001)], 2001)
    Rd, Rh = gpu.Reduced(csr), gpu.Reduced(csr, on_host=True)
    di, hi = Rd.info(), Rh.info()
    assert di["on_device"] == 1 and hi["on_device"] == 0
    for k in ("n", "d1_folded", "d1_hubs", "alive", "articulation_points", "blocks", "max_block", "block_slots",
              "block_edges", "components"):
        assert di[k] == hi[k], (case, k, di[k], hi[k])
    # vertices with live edges are the same; a tree component keeps one root,
    # which may be either end of its last edge
    cd, wd, vd = Rd.core_graph()
    ch, wh, vh = Rh.core_graph()
    kd, kh = np.diff(cd.row) > 0, np.diff(ch.row) > 0
    assert np.array_equal(vd[kd], vh[kh]) and np.array_equal(wd[kd], wh[kh])
    assert np.array_equal(np.sort(wd[~kd]), np.sort(wh[~kh]))
    for i, j in zip(np.nonzero(kd)[0], np.nonzero(kh)[0]):
        a, b = vd[cd.col[cd.row[i]:cd.row[i + 1]]], vh[ch.col[ch.row[j]:ch.row[j + 1]]]
        assert np.array_equal(np.sort(a), np.sort(b))
    (bd, bwd), (bh, bwh) = Rd.block_graph(), Rh.block_graph()
    assert bd.n == bh.n and np.array_equal(np.sort(bwd), np.sort(bwh))
    assert np.array_equal(Rd.cc(), Rh.cc())
    bcd, bch = Rd.bc(), Rh.bc()
    assert np.max(np.abs(bcd - bch) / np.maximum(np.abs(bch), 1.0)) < 1e-12


def test_device_reduction_rejects_bad_input(gpu):
    """gbc_reduce checks the entries on its device copy before any kernel
    indexes by them, with the host path's messages."""
    L = gpu.lib()
    h = C.c_void_p()
    row = np.array([0, 1, 2], np.int64)
    cases = [(row, np.array([0, 1], np.int32), 0, b"self-loop at vertex 0"),
             (row, np.array([1, 0], np.int32), 1, b"phantom slot 0 must have no edges"),
             (row, np.array([1, 2], np.int32), 0, b"col[1]=2 out of range"),
             (np.array([0, 2, 1, 2], np.int64), np.array([1, 0], np.int32), 0, b"row offsets decrease at 1")]
    for r, c, start, msg in cases:
        n = len(r) - 1
        for fn in (L.gbc_reduce, L.gbc_reduce_host):
            assert fn(r, c, n, start, C.byref(h)) == 1, msg
            assert msg in L.gbc_last_error(), (msg, L.gbc_last_error())


def test_c2_config_reduction_full_size(gpu, orc):
    """The D1-folding + AP-splitting configuration at full size: R-MAT scale
    18, edge factor 4 (a=.57, b=.19, c=.19) with 60K pendant paths of depth
    1-3 on random vertices (disconnected, isolated vertices).  Closeness of
    every vertex through the reduction equals the unreduced lane engine
    bit-exactly; betweenness through folding equals the unreduced Brandes
    within 1e-9; sampled vertices agree with the oracle."""
    csr = gpu.add_pendants(gpu.gen_rmat(18, 4, seed=18), 60000, 3, 2)
    assert 300_000 < csr.n < 450_000
    R = gpu.Reduced(csr)
    info = R.info()
    assert info["d1_folded"] > 60000 and info["components"] > 1000
    cc_red = R.cc()
    with gpu.Graph(csr) as G:
        cc_all = G.cc()
        assert np.array_equal(cc_red, cc_all)
        bc_all = G.bc()
    bc_red = R.bc()
    assert np.max(np.abs(bc_red - bc_all) / np.maximum(np.abs(bc_all), 1.0)) < 1e-9
    og = orc.Graph(csr.row, csr.col)
    pick = np.random.default_rng(2).choice(csr.n, 300, replace=False).astype(np.int32)
    assert np.array_equal(cc_red[pick], orc.cc(og, pick, nthreads=8))


def test_cached_lane_state_reused_and_released(gpu, orc):
    """Destroyed graphs leave their lane state in the library's cache; a new
    graph of the same size reuses it with identical results, and
    gbc_release_cached_memory returns it to the driver."""
    torch = pytest.importorskip("torch")
    csr = gpu.gen_rmat(14, 8, seed=11)
    src = np.arange(0, csr.n, 37, dtype=np.int32)[:256]
    gpu.check(gpu.lib().gbc_release_cached_memory())
    free0 = torch.cuda.mem_get_info()[0]
    with gpu.Graph(csr) as G:
        a = G.bc(src, lanes=256)
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 < free0 - (64 << 20)          # the engine's buffers stayed allocated (cached)
    with gpu.Graph(csr) as G:
        b = G.bc(src, lanes=256)
    assert np.array_equal(a, b)
    assert torch.cuda.mem_get_info()[0] >= free1 - (16 << 20)   # reused, not allocated again
    gpu.check(gpu.lib().gbc_release_cached_memory())
    assert torch.cuda.mem_get_info()[0] > free1 + (64 << 20)
    og = orc.Graph(csr.row, csr.col)
    ref, _ = orc.bc(og, src)
    assert np.max(np.abs(a - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-9


def test_autotune_choices_and_results(gpu, orc):
    """The autotuner returns valid settings, leaves explicit options alone,
    and later calls that use the tuned settings stay within tolerance of the
    oracle."""
    csr = gpu.gen_grid(60, 60, 0.05, seed=4)
    og = orc.Graph(csr.row, csr.col)
    src = np.arange(0, csr.n, 7, dtype=np.int32)[:256]
    ref, _ = orc.bc(og, src, scaled=True)
    with gpu.Graph(csr) as G:
        ch = G.autotune(src, light_steps=8)
        assert ch["light_steps"] == 8
        assert ch["sparse_lanes"] in (1, 2, 4) and ch["levels_per_graph"] in (16, 64)
        assert ch["lanes"] in (32, 64, 128, 256)
        got = G.bc(src)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-9
        ch2 = G.autotune(src)
        assert ch2["light_steps"] in (0, 8, 16, 32)
        assert ch2["block_threads"] in (128, 256, 512)
        assert np.array_equal(G.cc(src), orc.cc(og, src))
        ch3 = G.autotune(src, block_threads=512)
        assert ch3["block_threads"] == 512
        assert np.max(np.abs(G.bc(src) - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-9


def test_level_profile(gpu, orc):
    """gbc_graph_last_levels: the last batch's frontier entries per level add
    up to the run's frontier entries, the level count matches the oracle's
    deepest distance, and with one level kernel per graph there is one forward
    launch per level (plus the tail launch that finds the frontier empty) and
    one sweep launch per level below the deepest."""
    csr = gpu.gen_grid(20, 20, 0.05, seed=6)      # path counts stay exact (no wide re-run)
    src = np.arange(0, csr.n, 11, dtype=np.int32)[:32]
    with gpu.Graph(csr) as G:
        G.bc(src, lanes=32, levels_per_graph=1, sigma_mode=gpu.SIGMA_EXACT)
        st = G.stats()
        lv = G.levels()
    og = orc.Graph(csr.row, csr.col)
    depth = max(int(orc.sssp(og, s)[0].max()) for s in src) + 1
    assert len(lv["entries"]) == depth == st["levels"]
    assert int(lv["entries"].sum()) == st["frontier_entries"]
    assert lv["entries"][0] == 32 and np.all(lv["entries"] > 0)
    assert depth <= len(lv["fwd_ms"]) <= depth + 1 and len(lv["bwd_ms"]) == depth - 1
    assert np.all(lv["fwd_ms"] > 0) and np.all(lv["bwd_ms"] > 0)


def test_autotune_direction_share(gpu, orc):
    """On a small-world graph the autotuner also picks the closeness
    direction-switch share (or top-down only); closeness under the choice
    equals the oracle.  Out-of-range shapes and shares are refused."""
    csr = gpu.gen_rmat(14, 16, seed=3)
    og = orc.Graph(csr.row, csr.col)
    src = np.nonzero(np.diff(csr.row) > 0)[0][:512].astype(np.int32)
    with gpu.Graph(csr) as G:
        ch = G.autotune(src)
        assert ch["group_lanes"] == 128
        assert ch["bu_share"] in (0, 4, 8, 16, 32, 64)
        assert (ch["direction"] == 1) == (ch["bu_share"] == 0)
        assert np.array_equal(G.cc(src), orc.cc(og, src, nthreads=8))
        for bad in (dict(block_threads=384), dict(bu_share=-1), dict(bu_share=5000)):
            with pytest.raises(gpu.GbcError):
                G.cc(src, **bad)


def _canonical_csr(u, v, n):
    """Symmetric CSR without self-loops or repeats, rows ascending (numpy)."""
    a = np.concatenate([u, v]).astype(np.int64)
    b = np.concatenate([v, u]).astype(np.int64)
    keep = a != b
    key = np.unique(a[keep] * n + b[keep])
    row = np.concatenate([[0], np.cumsum(np.bincount(key // n, minlength=n))]).astype(np.int64)
    return row, (key % n).astype(np.int32)


@pytest.mark.parametrize("case", ["rmat", "grid", "er+noise", "empty", "datasets"])
def test_device_ingest_matches_host_csr(gpu, orc, datasets, case):
    """gbc_graph_from_edges builds on the GPU exactly the canonical CSR
    (symmetric, no self-loops or repeats, rows ascending) from edge lists in
    any order with repeats, reversed duplicates and self-loops."""
    rng = np.random.default_rng(3)
    if case == "datasets":
        cases = [gpu.read_edgelist(p) for p in datasets.values()]
    elif case == "rmat":
        cases = [gpu.gen_rmat(15, 8, seed=2)]
    elif case == "grid":
        cases = [gpu.gen_grid(80, 90, 0.1, seed=5, largest_only=False)]
    elif case == "er+noise":
        cases = [gpu.gen_er(5000, 6.0, seed=9)]
    else:
        cases = [gpu.CSR(np.zeros(11, np.int64), np.zeros(0, np.int32))]
    for csr in cases:
        u = np.repeat(np.arange(csr.n, dtype=np.int32), np.diff(csr.row))
        v = csr.col.copy()
        if case == "er+noise":
            extra = rng.integers(0, len(u), len(u) // 3)
            loops = np.arange(0, csr.n, 50, dtype=np.int32)
            u, v = np.concatenate([u, v[extra], loops]), np.concatenate([v, u[extra], loops])
        perm = rng.permutation(len(u))
        u, v = u[perm], v[perm]
        row, col = _canonical_csr(u, v, csr.n)
        if case in ("rmat", "grid", "er+noise"):
            assert np.array_equal(row, csr.row)      # generators already emit the canonical form
        with gpu.Graph.from_edges(u, v, csr.n) as G:
            got = G.csr
            assert got.n == csr.n
            assert np.array_equal(got.row, row) and np.array_equal(got.col, col)
            if 0 < csr.n <= 6000 and len(col):
                src_s = np.arange(0, csr.n, max(1, csr.n // 64), dtype=np.int32)
                og = orc.Graph(row, col)
                assert np.array_equal(G.cc(src_s), orc.cc(og, src_s))
    with pytest.raises(gpu.GbcError):
        gpu.Graph.from_edges(np.array([0, 5], np.int32), np.array([1, 12], np.int32), 10)


def test_device_side_csr_validation(gpu):
    """With a device present, the per-entry CSR checks run on the device copy:
    the same messages and first offending index as the host check, for the
    host-buffer and the device-pointer entry points, and offsets reported
    before neighbour ids."""
    torch = pytest.importorskip("torch")
    L = gpu.lib()
    n, m = 5000, 2_000_000
    row = np.linspace(0, m, n + 1).astype(np.int64)
    col = (np.arange(m) % n).astype(np.int32)
    h = C.c_void_p()
    gpu.check(L.gbc_graph_create(row, col, n, C.byref(h)))
    L.gbc_graph_destroy(h)
    bad = col.copy()
    bad[1_500_001] = n + 5
    bad[1_900_000] = -1
    assert L.gbc_graph_create(row, bad, n, C.byref(h)) == 1
    assert b"col[1500001]=5005 out of range" in L.gbc_last_error()
    rowbad = row.copy()
    rowbad[700] = rowbad[702] + 1
    assert L.gbc_graph_create(rowbad, bad, n, C.byref(h)) == 1
    assert b"decrease at 700" in L.gbc_last_error()
    for r, c, msg in ((row, bad, b"col[1500001]=5005 out of range"), (rowbad, col, b"decrease at 700")):
        d_row, d_col = torch.from_numpy(r).cuda(), torch.from_numpy(c).cuda()
        assert L.gbc_graph_create_device(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), n, m,
                                         C.byref(h)) == 1
        assert msg in L.gbc_last_error()
    d_row, d_col = torch.from_numpy(row).cuda(), torch.from_numpy(col).cuda()
    assert L.gbc_graph_create_device(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), n, m - 1,
                                     C.byref(h)) == 1
    assert b"row[n] != m" in L.gbc_last_error()


def test_set_device(gpu):
    L = gpu.lib()
    n = gpu.device_count()
    assert L.gbc_set_device(0) == 0
    assert L.gbc_set_device(n) == 1 and b"out of range" in L.gbc_last_error()
    assert L.gbc_set_device(-1) == 1


def test_dropin_driver_on_karate(gpu, datasets, tmp_path):
    """The C driver built against include/gbc_compat.h reproduces the
    reference's golden BC file for karate and its closeness outputs."""
    import subprocess
    exe = build_dropin_driver(gpu, tmp_path)
    prefix = str(tmp_path / "karate")
    r = subprocess.run([exe, datasets["karate.txt"], prefix], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    gold = np.loadtxt(os.path.join(GOLDEN, "karate_BC_Score.txt"), skiprows=1)
    with open(prefix + "_bc.txt") as f:
        assert f.readline().split() == ["1", "34"]
    got = np.loadtxt(prefix + "_bc.txt", skiprows=1)
    assert np.max(np.abs(got - gold) / np.maximum(gold, 1.0)) < 2e-6
    fx = fixture("karate.txt")
    assert np.array_equal(np.loadtxt(prefix + "_cc.txt", dtype=np.int64), fx["cc_ref"][1:])
    assert np.array_equal(np.loadtxt(prefix + "_d1ap.txt", dtype=np.int64), fx["d1ap_cc_ref"][1:])
    st = STRUCT["karate.txt"]
    assert r.stdout.split()[:6] == ["folded", str(st["d1"]), "hubs", str(st["hub"]), "aps", str(st["ap"])]


def test_reduce_from_device_arrays(gpu, datasets):
    """gbc_reduce_device on a CSR already on the device equals gbc_reduce on
    the same CSR from host memory, and rejects a bad CSR with the same message."""
    torch = pytest.importorskip("torch")
    L = gpu.lib()
    cases = [gpu.add_pendants(gpu.gen_rmat(14, 4, seed=5), 3000, 3, 9), gpu.read_edgelist(datasets["karate.txt"]),
             _chain_of_blocks(gpu)]
    for csr in cases:
        d_row = torch.from_numpy(csr.row).cuda()
        d_col = torch.from_numpy(csr.col).cuda()
        torch.cuda.synchronize()
        h = C.c_void_p()
        gpu.check(L.gbc_reduce_device(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), csr.n, csr.start,
                                      C.byref(h)))
        info = gpu.ReducedInfo()
        gpu.check(L.gbc_reduced_info_get(h, C.byref(info)))
        cc = np.zeros(csr.n, np.int64)
        gpu.check(L.gbc_cc_reduced(h, C.byref(gpu.options()), cc))
        gpu.check(L.gbc_reduced_destroy(h))
        R = gpu.Reduced(csr)
        assert info.as_dict() == R.info()
        assert np.array_equal(cc, R.cc())
    row = torch.tensor([0, 1, 2], dtype=torch.int64, device="cuda")
    col = torch.tensor([0, 1], dtype=torch.int32, device="cuda")   # self-loop at 0
    torch.cuda.synchronize()
    h = C.c_void_p()
    assert L.gbc_reduce_device(C.c_void_p(row.data_ptr()), C.c_void_p(col.data_ptr()), 2, 0, C.byref(h)) == 1
    assert b"self-loop at vertex 0" in L.gbc_last_error()

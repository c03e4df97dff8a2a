"""The CPU oracle pinned against the reference's golden vectors and its own
outputs (fixtures made by tests/golden/make_golden.py from the reference
compiled from source)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
STRUCT = json.load(open(os.path.join(GOLDEN, "structure.json")))
SMALL_BC = ["karate.txt", "dolphins.txt", "football.txt", "polbooks.txt", "testdata.txt", "testdata1.txt",
            "testdata2.txt", "ia-fb-messages.mtx"]


def fixture(name):
    return np.load(os.path.join(GOLDEN, name.split(".")[0] + ".npz"))


def test_karate_bc_golden_file(orc, datasets):
    """karate_BC_Score.txt: header 'start end', then one %f per vertex
    (Seq_Brandes/Brandes.c:2313-2322), reference semantics."""
    g = orc.load_edgelist(datasets["karate.txt"])
    gold = np.loadtxt(os.path.join(GOLDEN, "karate_BC_Score.txt"), skiprows=1)
    bc, novf = orc.bc(g, np.arange(1, g.N), orc.BC_REFERENCE)
    assert novf == 0
    assert len(gold) == g.N - 1
    assert np.max(np.abs(bc[1:] - gold) / np.maximum(gold, 1.0)) < 2e-6
    # textbook Brandes differs: 462.14 vs 792.49 for vertex 1
    bt, _ = orc.bc(g, np.arange(1, g.N), orc.BC_BRANDES)
    assert abs(bt[1] - 462.1428571428572) < 1e-9 and abs(bc[1] - 792.490476190476) < 1e-9


@pytest.mark.parametrize("name", SMALL_BC)
def test_bc_reference_semantics_vs_reference_fp32(orc, datasets, name):
    g = orc.load_edgelist(datasets[name])
    ref = fixture(name)["bc_ref_f32"].astype(np.float64)
    bc, _ = orc.bc(g, np.arange(g.start, g.N), orc.BC_REFERENCE, nthreads=4)
    # the reference accumulates sigma, delta and BC in FP32
    assert np.max(np.abs(bc[g.start:] - ref[g.start:]) / np.maximum(np.abs(ref[g.start:]), 1.0)) < 5e-5


LARGE_BC = ["tech-WHOIS.mtx", "ca-HepPh.mtx", "caida.mtx", "ia-email-EU.mtx"]


@pytest.mark.parametrize("name", LARGE_BC)
def test_bc_reference_semantics_vs_reference_fp32_large(orc, datasets, name):
    # 7.5K-32K sources: the reference's FP32 sigma, delta and BC sums drift from
    # the FP64 restatement by up to ~1.2e-3 relative (max) and ~8e-5 (99th
    # percentile), so these pins carry their own bounds.
    g = orc.load_edgelist(datasets[name])
    ref = fixture(name)["bc_ref_f32"].astype(np.float64)[g.start:]
    bc, _ = orc.bc(g, np.arange(g.start, g.N), orc.BC_REFERENCE, nthreads=8)
    err = np.abs(bc[g.start:] - ref) / np.maximum(np.abs(ref), 1.0)
    assert err.max() < 2e-3 and np.quantile(err, 0.99) < 2e-4


@pytest.mark.parametrize("name", SMALL_BC)
def test_bc_shared_traversal_reference_vs_oracle(orc, datasets, name):
    # The reference's computeBC_shareBased (Seq_Brandes/Brandes.c:374) derives a
    # neighbour's BFS DAG from the source's traversal; its sums are computeBC's
    # (reference semantics), so the same FP64 restatement pins it.
    g = orc.load_edgelist(datasets[name])
    ref = fixture(name)["bc_shared_ref_f32"].astype(np.float64)
    bc, _ = orc.bc(g, np.arange(g.start, g.N), orc.BC_REFERENCE, nthreads=4)
    assert np.max(np.abs(bc[g.start:] - ref[g.start:]) / np.maximum(np.abs(ref[g.start:]), 1.0)) < 5e-5


def test_brandes_semantics_vs_networkx(orc, datasets):
    nx = pytest.importorskip("networkx")
    for name in ["karate.txt", "dolphins.txt", "testdata1.txt", "testdata2.txt"]:
        g = orc.load_edgelist(datasets[name])
        G = nx.Graph()
        G.add_nodes_from(range(g.start, g.N))
        for v in range(g.start, g.N):
            for e in range(g.row[v], g.row[v + 1]):
                G.add_edge(v, int(g.col[e]))
        nb = nx.betweenness_centrality(G, normalized=False)
        bc, _ = orc.bc(g, np.arange(g.start, g.N), orc.BC_BRANDES)
        for v in range(g.start, g.N):
            assert abs(2 * nb[v] - bc[v]) < 1e-9 * max(1.0, bc[v])


@pytest.mark.parametrize("name", sorted(STRUCT))
def test_cc_and_structure_vs_reference(orc, datasets, name):
    g = orc.load_edgelist(datasets[name])
    fx = fixture(name)
    cc = orc.cc(g, np.arange(g.start, g.N), nthreads=4)
    assert np.array_equal(cc, fx["cc_ref"][g.start:])
    # the reference's release path (D1 + AP, shared BFS) agrees on these connected inputs
    assert np.array_equal(cc, fx["d1ap_cc_ref"][g.start:])
    st = STRUCT[name]
    f = orc.d1_fold(g)
    assert (f["n_folded"], f["n_hub"]) == (st["d1"], st["hub"])
    _, nap = orc.articulation_points(g)
    assert nap == st["ap"]
    full = np.zeros(g.N, np.int64)
    full[g.start:] = cc
    assert np.array_equal(orc.d1_cc(g, fix_components=True)[g.start:], cc)
    shared, runs = orc.cc_shared(g)
    assert np.array_equal(shared[g.start:], cc)
    assert runs <= g.N - g.start
    apcc, _ = orc.ap_cc(g)
    is_ap, _ = orc.articulation_points(g)
    assert np.array_equal(apcc[is_ap], full[is_ap])


def _edges_graph(orc, n, edges):
    row = np.zeros(n + 1, np.int64)
    adj = [[] for _ in range(n)]
    for u, v in edges:
        adj[u].append(v)
        adj[v].append(u)
    col = []
    for v in range(n):
        row[v + 1] = row[v] + len(adj[v])
        col += adj[v]
    return orc.Graph(row, np.array(col, np.int32), start=1)


def test_d1_recovery_defect_on_disconnected_graph(orc):
    """Edge list '8 7 / 1 2 / 2 3 / 3 1 / 3 4 / 5 6 / 6 7 / 7 5': triangle
    1-2-3 with pendant 4, triangle 5-6-7, vertex 8 isolated (1-based).  The
    reference's D1 recovery uses the global vertex count (8) and gives
    CC[4] = 9; plain BFS gives 5 (the component-size fix)."""
    g = _edges_graph(orc, 9, [(1, 2), (2, 3), (3, 1), (3, 4), (5, 6), (6, 7), (7, 5)])
    plain = orc.cc(g, np.arange(1, 9))
    assert plain[3] == 5
    assert orc.d1_cc(g, fix_components=False)[4] == 9
    assert np.array_equal(orc.d1_cc(g, fix_components=True)[1:], plain)


def test_sigma_overflow_detected_and_scaled_delta(orc):
    # 40x40 grid: corner-to-corner path count C(78,39) > 2^64
    n = 40 * 40
    edges = []
    for r in range(40):
        for c in range(40):
            v = r * 40 + c
            if c + 1 < 40:
                edges.append((v, v + 1))
            if r + 1 < 40:
                edges.append((v, v + 40))
    row = np.zeros(n + 1, np.int64)
    adj = [[] for _ in range(n)]
    for u, v in edges:
        adj[u].append(v)
        adj[v].append(u)
    col = []
    for v in range(n):
        row[v + 1] = row[v] + len(adj[v])
        col += adj[v]
    g = orc.Graph(row, np.array(col, np.int32))
    dist, sig, ovf, npred = orc.sssp(g, 0)
    assert ovf[n - 1] and not ovf[1]
    assert dist[n - 1] == 78
    assert int(sig[40 * 5 + 5]) == 252   # C(10,5)
    # where exact counts fit, the level-normalised FP64 form gives the same dependencies
    small = _edges_graph(orc, 8, [(1, 2), (2, 3), (3, 1), (3, 4), (5, 6), (6, 7), (7, 5)])
    a, _ = orc.bc(small, np.arange(1, 8), scaled=False)
    b, _ = orc.bc(small, np.arange(1, 8), scaled=True)
    assert np.allclose(a, b, rtol=1e-12, atol=0)


def test_threaded_oracle_matches_serial(orc, datasets):
    g = orc.load_edgelist(datasets["ia-fb-messages.mtx"])
    src = np.arange(g.start, g.N)
    a, _ = orc.bc(g, src, nthreads=1)
    b, _ = orc.bc(g, src, nthreads=6)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
    assert np.array_equal(orc.cc(g, src, nthreads=1), orc.cc(g, src, nthreads=5))


@pytest.mark.parametrize("scale,ef,permute", [(12, 8, False), (16, 16, True)])
def test_oracle_rmat_generator_equals_product(gbc, orc, scale, ef, permute):
    """bench.py's CPU legs build the R-MAT workload with the oracle's
    restatement of the generator, so that the reference arm never loads the
    product library; both generators must give the same arrays and the same
    sampled sources."""
    import bench
    a = orc.gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed=1, permute=permute)
    b = gbc.gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed=1, permute=permute)
    assert np.array_equal(a.row, b.row) and np.array_equal(a.col, b.col)
    assert np.array_equal(bench.sample_sources(a.row, 1024), bench.sample_sources(b.row, 1024))


def test_reference_arm_line_without_the_library(tmp_path):
    """bench.py --impl reference prints one JSON line with the fields the
    measurement contract asks for, timing the oracle on the host cores, and
    never maps libgbc.so into its process (it builds the R-MAT graph with the
    oracle's restatement of the generator)."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    probe = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--scale', '12', '--edge-factor', '8', "
        "'--k', '256', '--steps', '1', '--warmup', '1']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit:\n"
        "    pass\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('LIBGBC_MAPPED' if 'libgbc.so' in maps else 'LIBGBC_ABSENT')\n")
    r = subprocess.run([sys.executable, "-c", probe], cwd=root, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert lines[-1] == "LIBGBC_ABSENT"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["unit"] == "GTEPS" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0

"""The C-ABI library on CPU: it loads, exports every symbol the public headers
declare, validates arguments before touching a device, and its host-side
parts (generators, edge-list reader, D1/block reduction assembly) agree with
the oracle.  No device compute happens here."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    names = set()
    for h in ("gbc.h", "gbc_compat.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", txt, flags=re.M):
            name = m.group(1)
            if name not in ("if", "for", "while", "sizeof", "return"):
                names.add(name)
    return sorted(names)


def test_exports_every_declared_symbol(gbc):
    L = gbc.lib()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_options(gbc):
    assert b"sm_103a" in gbc.lib().gbc_version()
    o = gbc.options()
    assert (o.semantics, o.delta_precision, o.sigma_mode, o.engine, o.lanes, o.sparse_lanes, o.light_steps) == (0, 1, 0, 0, 0, -1, -1)
    assert gbc.device_count() >= 0


def test_argument_validation_before_device(gbc):
    L = gbc.lib()
    h = C.c_void_p()
    row = np.array([0, 1, 2], np.int64)
    bad = np.array([1, 5], np.int32)          # neighbour id out of range
    assert L.gbc_graph_create(row, bad, 2, C.byref(h)) == 1
    assert b"out of range" in L.gbc_last_error()
    dec = np.array([0, 2, 1], np.int64)       # decreasing offsets
    assert L.gbc_graph_create(dec, np.array([1, 0], np.int32), 2, C.byref(h)) == 1
    assert L.gbc_bc(None, None, 0, None, np.zeros(1)) == 1
    n = C.c_int32()
    assert L.gbc_graph_last_levels(None, None, 0, None, None, 0, C.byref(n), None, None) == 1
    sz = C.c_size_t()
    assert L.gbc_server_request_bytes(None, 0, 0, C.byref(sz), C.byref(sz)) == 1
    if gbc.device_count() == 0:
        ok = np.array([1, 0], np.int32)
        assert L.gbc_graph_create(row, ok, 2, C.byref(h)) == 9   # GBC_ERR_NO_DEVICE


def _check_csr(csr):
    n = csr.n
    assert csr.row[0] == 0 and np.all(np.diff(csr.row) >= 0)
    src = np.repeat(np.arange(n), np.diff(csr.row))
    assert np.all(src != csr.col), "self-loop"
    key = src.astype(np.int64) * n + csr.col
    rkey = csr.col.astype(np.int64) * n + src
    assert np.array_equal(np.sort(key), np.sort(rkey)), "not symmetric"
    for v in range(0, n, max(1, n // 200)):
        r = csr.col[csr.row[v]:csr.row[v + 1]]
        assert np.all(np.diff(r) > 0), "row not sorted/deduplicated"


def test_generators(gbc):
    ba = gbc.gen_ba(4096, 4, 1)
    assert ba.n == 4096 and ba.m == 2 * (4 + 4 * (4096 - 5))
    _check_csr(ba)
    assert np.array_equal(gbc.gen_ba(4096, 4, 1).col, ba.col)
    assert not np.array_equal(gbc.gen_ba(4096, 4, 2).col, ba.col)
    rm = gbc.gen_rmat(12, 8, seed=3)
    assert rm.n == 4096
    _check_csr(rm)
    assert np.array_equal(gbc.gen_rmat(12, 8, seed=3).col, rm.col)
    gr = gbc.gen_grid(64, 64, 0.05, seed=3)
    _check_csr(gr)
    assert gr.n <= 4096 and gr.m <= 2 * (2 * 64 * 63)
    full = gbc.gen_grid(10, 12, 0.0, seed=1)
    assert full.n == 120 and full.m == 2 * (10 * 11 + 12 * 9)
    er = gbc.gen_er(1000, 4.0, 7)
    _check_csr(er)
    pend = gbc.add_pendants(er, 100, 3, 5)
    _check_csr(pend)
    assert 1100 <= pend.n <= 1300 and pend.m == er.m + 2 * (pend.n - er.n)


def test_reader_matches_oracle_reader(gbc, orc, datasets):
    for name, path in datasets.items():
        a = gbc.read_edgelist(path)
        b = orc.load_edgelist(path)
        assert (a.n, a.start) == (b.N, b.start), name
        assert np.array_equal(a.row, b.row) and np.array_equal(a.col, b.col), name


def _reduced_cc_host(gbc, orc, csr):
    """Block graph from the library, its weighted sums from the oracle, the
    library's host assembly: the whole reduction except the device BFS."""
    R = gbc.Reduced(csr, on_host=True)
    bg, w = R.block_graph()
    ob = orc.Graph(bg.row, bg.col)
    D = orc.cc(ob, np.arange(bg.n), w=w.astype(np.int64), ff=np.zeros(bg.n, np.int64), nthreads=4)
    return R, R.assemble_cc(D)


def test_reduction_host_logic_on_reference_datasets(gbc, orc, datasets):
    struct = json.load(open(os.path.join(GOLDEN, "structure.json")))
    for name, path in datasets.items():
        csr = gbc.read_edgelist(path)
        og = orc.Graph(csr.row, csr.col, csr.start)
        ref = np.zeros(csr.n, np.int64)
        ref[csr.start:] = orc.cc(og, np.arange(csr.start, csr.n), nthreads=4)
        R, got = _reduced_cc_host(gbc, orc, csr)
        assert np.array_equal(got, ref), name
        info = R.info()
        st = struct[name]
        assert (info["d1_folded"], info["d1_hubs"], info["articulation_points"]) == (st["d1"], st["hub"], st["ap"])


@pytest.mark.parametrize("case", ["rmat+pendants", "sparse-er+pendants", "grid-holes", "path", "star", "trees"])
def test_reduction_host_logic_disconnected(gbc, orc, case):
    if case == "rmat+pendants":
        csr = gbc.add_pendants(gbc.gen_rmat(11, 4, seed=5), 500, 3, 9)
    elif case == "sparse-er+pendants":
        csr = gbc.add_pendants(gbc.gen_er(2000, 1.5, seed=5), 300, 3, 9)
    elif case == "grid-holes":
        csr = gbc.gen_grid(30, 30, 0.3, seed=2, largest_only=False)
    elif case == "path":
        n = 50
        row = np.concatenate([[0], np.cumsum([1] + [2] * (n - 2) + [1])]).astype(np.int64)
        col = []
        for v in range(n):
            col += ([v - 1] if v > 0 else []) + ([v + 1] if v < n - 1 else [])
        csr = gbc.CSR(row, np.array(col, np.int32))
    elif case == "star":
        n = 30
        row = np.array([0, n - 1] + list(range(n, 2 * n - 1)), np.int64)
        col = np.array(list(range(1, n)) + [0] * (n - 1), np.int32)
        csr = gbc.CSR(row, col)
    else:   # a forest of pendant paths on isolated vertices
        base = gbc.CSR(np.zeros(41, np.int64), np.zeros(0, np.int32))
        csr = gbc.add_pendants(base, 60, 3, 4)
    og = orc.Graph(csr.row, csr.col, csr.start)
    ref = orc.cc(og, np.arange(csr.n), nthreads=4)
    _, got = _reduced_cc_host(gbc, orc, csr)
    assert np.array_equal(got, ref)


def test_reduce_rejects_bad_input(gbc):
    L = gbc.lib()
    h = C.c_void_p()
    row = np.array([0, 1, 2], np.int64)
    loop = np.array([0, 1], np.int32)   # self-loop at 0
    assert L.gbc_reduce_host(row, loop, 2, 0, C.byref(h)) == 1
    assert b"self-loop at vertex 0" in L.gbc_last_error()
    ok = np.array([1, 0], np.int32)
    assert L.gbc_reduce_host(row, ok, 2, 1, C.byref(h)) == 1   # phantom slot with edges
    if gbc.device_count() == 0:
        # the device reduction checks its argument header, then needs a device
        assert L.gbc_reduce(row, np.array([1, 5], np.int32), 2, 0, C.byref(h)) == 9
        assert L.gbc_reduce(row, ok, 2, 7, C.byref(h)) == 1


def _weighted_brandes(csr, w):
    """Reach-weighted Brandes on a small CSR (pure Python; test helper)."""
    from collections import deque
    n = csr.n
    bc = np.zeros(n)
    for s in range(n):
        dist = [-1] * n
        sig = [0] * n
        dist[s] = 0
        sig[s] = 1
        order = []
        q = deque([s])
        while q:
            v = q.popleft()
            order.append(v)
            for e in range(csr.row[v], csr.row[v + 1]):
                x = int(csr.col[e])
                if dist[x] < 0:
                    dist[x] = dist[v] + 1
                    q.append(x)
                if dist[x] == dist[v] + 1:
                    sig[x] += sig[v]
        delta = [0.0] * n
        for v in reversed(order):
            acc = 0.0
            for e in range(csr.row[v], csr.row[v + 1]):
                x = int(csr.col[e])
                if dist[x] == dist[v] + 1:
                    acc += (w[x] + delta[x]) / sig[x]
            delta[v] = sig[v] * acc
            if v != s:
                bc[v] += w[s] * delta[v]
    return bc


@pytest.mark.parametrize("case", ["karate", "testdata1", "pendants", "forest"])
def test_reduced_bc_host_logic(gbc, orc, datasets, case):
    """Folding pair counts + reach-weighted Brandes on the core (here on the
    CPU) reproduce plain Brandes betweenness of the unreduced graph."""
    if case == "karate":
        csr = gbc.read_edgelist(datasets["karate.txt"])
    elif case == "testdata1":
        csr = gbc.read_edgelist(datasets["testdata1.txt"])
    elif case == "pendants":
        csr = gbc.add_pendants(gbc.gen_er(150, 2.5, seed=3), 80, 3, 4)
    else:
        base = gbc.CSR(np.zeros(21, np.int64), np.zeros(0, np.int32))
        csr = gbc.add_pendants(base, 30, 3, 4)
    og = orc.Graph(csr.row, csr.col, csr.start)
    ref, _ = orc.bc(og, np.arange(csr.start, csr.n), semantics=orc.BC_BRANDES)
    R = gbc.Reduced(csr, on_host=True)
    core, w, vert = R.core_graph()
    info = R.info()
    assert len(vert) == info["alive"] and int(w.sum()) == csr.n - csr.start   # reach covers every vertex once
    got = R.assemble_bc(_weighted_brandes(core, w))
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-9


def test_validation_reports_first_bad_entry(gbc):
    """Large CSRs are validated by several threads; the error still names the
    first offending entry."""
    L = gbc.lib()
    n = 1000
    m = 400_000
    row = np.linspace(0, m, n + 1).astype(np.int64)
    col = (np.arange(m) % n).astype(np.int32)
    col[150_001] = n + 5
    col[390_000] = -1
    h = C.c_void_p()
    assert L.gbc_graph_create(row, col, n, C.byref(h)) == 1
    assert b"col[150001]" in L.gbc_last_error()
    rowbad = row.copy()
    rowbad[700] = rowbad[702] + 1
    assert L.gbc_graph_create(rowbad, np.zeros(m, np.int32), n, C.byref(h)) == 1
    assert b"decrease at 700" in L.gbc_last_error()


def test_score_file_matches_reference_layout(gbc, orc, datasets, tmp_path):
    """gbc_write_scores writes the reference's BC_Score.txt layout: karate BC
    (reference semantics, from the oracle) against the reference's golden
    file, line by line."""
    csr = gbc.read_edgelist(datasets["karate.txt"])
    og = orc.Graph(csr.row, csr.col, csr.start)
    bc, _ = orc.bc(og, np.arange(csr.start, csr.n), semantics=orc.BC_REFERENCE)
    out = tmp_path / "BC_Score.txt"
    gbc.write_scores(str(out), bc, csr.start, csr.n - 1)
    got = out.read_text().splitlines()
    gold = open(os.path.join(GOLDEN, "karate_BC_Score.txt")).read().splitlines()
    assert got[0] == gold[0] == "1 34" and len(got) == len(gold)
    for a, b in zip(got[1:], gold[1:]):
        assert len(a.split(".")[1]) == 6                 # "%f"
        assert abs(float(a) - float(b)) <= 2e-6 * max(1.0, float(b))
    gbc.write_scores(str(out), bc, csr.start, csr.start, append=True)
    assert out.read_text().splitlines()[-2:] == ["1 1", got[1]]


def test_set_device_without_gpu(gbc):
    if gbc.device_count() > 0:
        pytest.skip("a device is visible")
    assert gbc.lib().gbc_set_device(0) == 9    # GBC_ERR_NO_DEVICE

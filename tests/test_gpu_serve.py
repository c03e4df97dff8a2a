"""GPU serving: continuous batching over device-resident graphs.  Requests
that arrive while others run share lane batches; every result equals the
same request run alone (closeness exactly, betweenness within 1e-9
relative), and deadlines, cancellation and admission behave."""
import ctypes as C
import random
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-9


class Server:
    def __init__(self, gbc, budget=0, max_lanes=0, max_inflight=0, workers=0):
        self.g = gbc
        self.L = gbc.lib()
        cfg = gbc.ServerConfig()
        cfg.hbm_budget_bytes = budget
        cfg.max_lanes = max_lanes
        cfg.max_inflight = max_inflight
        cfg.workers = workers
        self.h = C.c_void_p()
        gbc.check(self.L.gbc_server_create(C.byref(cfg), C.byref(self.h)))
        self.n = {}

    def add(self, csr):
        gid = C.c_int32()
        self.g.check(self.L.gbc_server_add_graph(self.h, csr.row, csr.col, csr.n, C.byref(gid)))
        self.n[gid.value] = csr.n
        return gid.value

    def submit(self, gid, kind, k=0, seed=0, deadline_ms=0.0, **opt):
        rid = C.c_int64()
        self.g.check(self.L.gbc_server_submit(self.h, gid, kind, k, seed, C.byref(self.g.options(**opt)),
                                              deadline_ms, C.byref(rid)))
        return rid.value

    def wait(self, rid, timeout_ms=120000.0):
        st = C.c_int32()
        self.g.check(self.L.gbc_server_wait(self.h, rid, timeout_ms, C.byref(st)))
        return st.value

    def fetch(self, rid, gid):
        n = self.n[gid]
        bc = np.zeros(n, np.float64)
        cc = np.zeros(n, np.int64)
        lat = C.c_double()
        st = self.L.gbc_server_fetch(self.h, rid, bc.ctypes.data_as(C.c_void_p), cc.ctypes.data_as(C.c_void_p),
                                     C.byref(lat))
        return st, bc, cc, lat.value

    def sources(self, rid):
        k = C.c_int32()
        self.g.check(self.L.gbc_server_sources(self.h, rid, None, 0, C.byref(k)))
        out = np.zeros(k.value, np.int32)
        self.g.check(self.L.gbc_server_sources(self.h, rid, out.ctypes.data_as(C.c_void_p), k.value, C.byref(k)))
        return out

    def counters(self):
        v = [C.c_int64() for _ in range(4)] + [C.c_double()]
        self.g.check(self.L.gbc_server_counters(self.h, *[C.byref(x) for x in v]))
        return dict(completed=v[0].value, batches=v[1].value, shared=v[2].value, edges=v[3].value,
                    busy_ms=v[4].value)

    def close(self):
        self.L.gbc_server_destroy(self.h)


def relerr(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.fixture(scope="module")
def graphs(gpu):
    return [gpu.gen_ba(2000, 3, 1), gpu.gen_grid(30, 30, 0.05, seed=3), gpu.gen_rmat(11, 8, seed=2),
            gpu.gen_er(1500, 6.0, seed=4)]


def run_alone(gpu, csr, kind, k, seed, sem):
    S = Server(gpu)
    gid = S.add(csr)
    rid = S.submit(gid, kind, k, seed, semantics=sem)
    assert S.wait(rid) == gpu.REQ_DONE
    st, bc, cc, _ = S.fetch(rid, gid)
    assert st == 0
    S.close()
    return bc, cc


def test_mixed_stream_equals_alone(gpu, orc, graphs):
    S = Server(gpu, max_lanes=256)
    gids = [S.add(g) for g in graphs]
    rng = random.Random(5)
    plan = []
    for i in range(24):
        gi = rng.randrange(len(graphs))
        kind = rng.choice([gpu.Q_CC, gpu.Q_BC_SAMPLED, gpu.Q_BC_SAMPLED, gpu.Q_BC])
        k = rng.choice([64, 300]) if kind == gpu.Q_BC_SAMPLED else 0
        if kind == gpu.Q_BC and graphs[gi].n > 1200:
            kind, k = gpu.Q_BC_SAMPLED, 1024
        plan.append((gi, kind, k, 100 + i, rng.choice([0, 1])))
    rids = [None] * len(plan)

    def client(lo, hi):
        for j in range(lo, hi):
            gi, kind, k, seed, sem = plan[j]
            rids[j] = S.submit(gids[gi], kind, k, seed, semantics=sem)
            time.sleep(rng.random() * 0.01)

    th = [threading.Thread(target=client, args=(a, a + 6)) for a in range(0, 24, 6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    results = []
    for j, rid in enumerate(rids):
        assert S.wait(rid) == gpu.REQ_DONE
        results.append(S.fetch(rid, gids[plan[j][0]]))
    # whether the stream above shares batches depends on its timing; four requests submitted
    # back to back on one graph share at least the batch after the first one's
    burst = [S.submit(gids[0], gpu.Q_BC_SAMPLED, 64, 900 + i) for i in range(4)]
    for r in burst:
        assert S.wait(r) == gpu.REQ_DONE
        assert S.fetch(r, gids[0])[0] == 0
    c = S.counters()
    S.close()
    assert c["completed"] == len(plan) + len(burst)
    assert c["shared"] > 0, "no lane batch carried more than one request"
    lats = [r[3] for r in results]
    assert all(l > 0 for l in lats)
    for j, (gi, kind, k, seed, sem) in enumerate(plan):
        st, bc, cc, _ = results[j]
        assert st == 0
        abc, acc = run_alone(gpu, graphs[gi], kind, k, seed, sem)
        if kind == gpu.Q_CC:
            assert np.array_equal(cc, acc)
            og = orc.Graph(graphs[gi].row, graphs[gi].col)
            assert np.array_equal(cc, orc.cc(og, np.arange(graphs[gi].n)))
        else:
            assert relerr(bc, abc) < TOL, (j, plan[j])
    # exact-BC requests checked against the oracle over all sources
    for j, (gi, kind, k, seed, sem) in enumerate(plan):
        if kind != gpu.Q_BC:
            continue
        og = orc.Graph(graphs[gi].row, graphs[gi].col)
        ref, _ = orc.bc(og, np.arange(graphs[gi].n), semantics=sem, nthreads=8)
        assert relerr(results[j][1], ref) < TOL


def test_deadline_cancel_and_unknown(gpu, graphs):
    S = Server(gpu, max_lanes=32)
    gid = S.add(graphs[0])
    slow = S.submit(gid, gpu.Q_BC, deadline_ms=1.0)      # 2000 sources in 32-lane batches: cannot finish in 1 ms
    assert S.wait(slow) == gpu.REQ_FAILED
    st, _, _, _ = S.fetch(slow, gid)
    assert st == 8   # GBC_ERR_TIMEOUT
    r2 = S.submit(gid, gpu.Q_BC)
    S.g.check(S.L.gbc_server_cancel(S.h, r2))
    assert S.wait(r2) == gpu.REQ_CANCELLED
    st = C.c_int32()
    assert S.L.gbc_server_poll(S.h, 987654, C.byref(st)) == 6   # GBC_ERR_NOT_FOUND
    rid = C.c_int64()
    assert S.L.gbc_server_submit(S.h, 99, gpu.Q_CC, 0, 0, None, 0.0, C.byref(rid)) == 6
    ok = S.submit(gid, gpu.Q_BC_SAMPLED, 40, 7)
    assert S.wait(ok) == gpu.REQ_DONE
    S.close()


def test_admission_under_small_budget(gpu, orc, graphs):
    # a budget that holds only a narrow engine for one graph at a time
    S = Server(gpu, budget=64 << 20, max_lanes=1024)
    gids = [S.add(g) for g in graphs[:3]]
    rids = [(g, S.submit(g, gpu.Q_CC)) for g in gids]
    for g, r in rids:
        assert S.wait(r) == gpu.REQ_DONE
        st, _, cc, _ = S.fetch(r, g)
        assert st == 0
        csr = graphs[gids.index(g)]
        og = orc.Graph(csr.row, csr.col)
        assert np.array_equal(cc, orc.cc(og, np.arange(csr.n)))
    S.close()


def request_bytes(S, gid, kind):
    res, eng = C.c_size_t(), C.c_size_t()
    S.g.check(S.L.gbc_server_request_bytes(S.h, gid, kind, C.byref(res), C.byref(eng)))
    return res.value, eng.value


def test_admission_by_device_footprint(gpu, orc, graphs):
    """A budget that holds one exact-BC request (result vector + the graph's
    narrowest engine) but not two: the second waits, queued, while the first
    one's result is held, is admitted once it is fetched, and both equal the
    oracle.  A request that could never fit fails with GBC_ERR_NOMEM."""
    g = graphs[3]
    probe = Server(gpu)
    gid0 = probe.add(g)
    res, eng = request_bytes(probe, gid0, gpu.Q_BC)
    assert res == 8 * g.n and eng > 0
    assert request_bytes(probe, gid0, gpu.Q_CC)[0] == 0
    probe.close()
    S = Server(gpu, budget=eng + res + res // 2, workers=1)
    gid = S.add(g)
    r1 = S.submit(gid, gpu.Q_BC)
    r2 = S.submit(gid, gpu.Q_BC)
    assert S.wait(r1) == gpu.REQ_DONE
    time.sleep(0.3)
    st = C.c_int32()
    S.g.check(S.L.gbc_server_poll(S.h, r2, C.byref(st)))
    assert st.value == gpu.REQ_QUEUED, "the second request was admitted past the budget"
    st1, bc1, _, _ = S.fetch(r1, gid)
    assert st1 == 0
    assert S.wait(r2) == gpu.REQ_DONE
    st2, bc2, _, _ = S.fetch(r2, gid)
    assert st2 == 0
    S.close()
    ref, _ = orc.bc(orc.Graph(g.row, g.col), np.arange(g.n), nthreads=8)
    assert relerr(bc1, ref) < TOL and relerr(bc2, ref) < TOL
    tiny = Server(gpu, budget=eng + res - 1)
    gid = tiny.add(g)
    r = tiny.submit(gid, gpu.Q_BC)
    assert tiny.wait(r) == gpu.REQ_FAILED
    assert tiny.fetch(r, gid)[0] == 3   # GBC_ERR_NOMEM
    r = tiny.submit(gid, gpu.Q_CC)       # closeness results live on the host: it fits
    assert tiny.wait(r) == gpu.REQ_DONE
    tiny.close()


def test_c5_size_mixed_equals_alone(gpu, graphs):
    """Serving at the size of the serving mix: a k=1024 sampled-BC request on
    an R-MAT scale-20 graph (1M vertices) submitted among small requests on
    other graphs gives the same result as alone, and the same as a graph
    handle's gbc_bc over the request's own sources."""
    big = gpu.gen_rmat(20, 16, seed=21)
    S = Server(gpu)
    gb = S.add(big)
    small = [S.add(g) for g in graphs]
    rng = random.Random(9)
    pre = [(gi, S.submit(small[gi], gpu.Q_BC_SAMPLED, 256, 500 + j)) for j, gi in
           enumerate(rng.choice(range(len(graphs))) for _ in range(6))]
    rb = S.submit(gb, gpu.Q_BC_SAMPLED, 1024, 77)
    src = S.sources(rb)
    post = [(gi, S.submit(small[gi], gpu.Q_CC if j % 2 else gpu.Q_BC_SAMPLED, 64, 600 + j)) for j, gi in
            enumerate(rng.choice(range(len(graphs))) for _ in range(6))]
    for gi, r in pre + post:
        assert S.wait(r) == gpu.REQ_DONE
        assert S.fetch(r, small[gi])[0] == 0
    assert S.wait(rb, 600000.0) == gpu.REQ_DONE
    st, mixed, _, _ = S.fetch(rb, gb)
    assert st == 0
    S.close()
    alone, _ = run_alone(gpu, big, gpu.Q_BC_SAMPLED, 1024, 77, 0)
    assert relerr(mixed, alone) < TOL
    with gpu.Graph(big) as h:
        direct = h.bc(src)
    assert relerr(mixed, direct) < TOL
    assert np.count_nonzero(mixed) > big.n // 4


def test_worker_count(gpu, orc, graphs):
    """One worker and eight workers give the same results on the same
    stream; out-of-range worker counts are rejected."""
    cfg = gpu.ServerConfig()
    cfg.workers = 17
    h = C.c_void_p()
    assert gpu.lib().gbc_server_create(C.byref(cfg), C.byref(h)) == 1   # GBC_ERR_ARG
    out = {}
    for w in (1, 8):
        S = Server(gpu, max_lanes=128, workers=w)
        gids = [S.add(g) for g in graphs]
        rids = [(gi, S.submit(gids[gi], gpu.Q_BC_SAMPLED, 200, 40 + gi)) for gi in range(len(graphs))]
        rids += [(1, S.submit(gids[1], gpu.Q_CC))]
        res = []
        for gi, rid in rids:
            assert S.wait(rid) == gpu.REQ_DONE
            st, bc, cc, _ = S.fetch(rid, gids[gi])
            assert st == 0
            res.append((bc, cc))
        S.close()
        out[w] = res
    for (b1, c1), (b8, c8) in zip(out[1], out[8]):
        assert relerr(b8, b1) < TOL
        assert np.array_equal(c8, c1)
    og = orc.Graph(graphs[1].row, graphs[1].col)
    assert np.array_equal(out[8][-1][1], orc.cc(og, np.arange(graphs[1].n)))


def spread_over(gpu, csr, extra, seed):
    """csr's vertices moved to random ids among csr.n + extra; the other ids are isolated."""
    N = csr.n + extra
    p = np.random.default_rng(seed).permutation(N)[:csr.n]
    a = p[np.repeat(np.arange(csr.n), np.diff(csr.row))]
    b = p[csr.col]
    order = np.lexsort((b, a))
    row = np.zeros(N + 1, np.int64)
    np.add.at(row, a + 1, 1)
    return gpu.CSR(np.cumsum(row), b[order].astype(np.int32))


def test_isolated_sources_take_no_lane(gpu, orc):
    """Sources without edges reach nothing: they are listed after the others,
    take no lane, and the results still equal the oracle over every source.
    A request whose sources are all isolated completes at submission with a
    zero result."""
    g = spread_over(gpu, gpu.gen_ba(600, 3, 8), 424, 2)
    iso = np.nonzero(np.diff(g.row) == 0)[0]
    assert len(iso) == 424
    og = orc.Graph(g.row, g.col)
    S = Server(gpu, max_lanes=128)
    gid = S.add(g)
    r_cc = S.submit(gid, gpu.Q_CC)
    r_bc = S.submit(gid, gpu.Q_BC)
    r_s = S.submit(gid, gpu.Q_BC_SAMPLED, 300, 5)
    src = S.sources(r_s)
    assert len(src) == 300 and len(S.sources(r_bc)) == g.n
    flag = np.isin(src, iso)
    k_edge = int((~flag).sum())
    assert 0 < k_edge < 300 and not flag[:k_edge].any() and flag[k_edge:].all()
    for r in (r_cc, r_bc, r_s):
        assert S.wait(r) == gpu.REQ_DONE
    c = S.counters()
    # exact requests run the 600 vertices with edges in 128-lane batches (8 each if the 424
    # isolated ones took lanes), the sample its k_edge sources
    assert c["batches"] <= 2 * 5 + (k_edge + 127) // 128
    st, _, cc, _ = S.fetch(r_cc, gid)
    assert st == 0 and np.array_equal(cc, orc.cc(og, np.arange(g.n)))
    st, bc, _, _ = S.fetch(r_bc, gid)
    ref, _ = orc.bc(og, np.arange(g.n), nthreads=8)
    assert st == 0 and relerr(bc, ref) < TOL
    st, bs, _, _ = S.fetch(r_s, gid)
    ref, _ = orc.bc(og, src, nthreads=8)
    assert st == 0 and relerr(bs, ref) < TOL
    S.close()
    # one edge among 1000 vertices: a one-source sample almost surely draws an isolated vertex
    two = spread_over(gpu, gpu.CSR(np.array([0, 1, 2], np.int64), np.array([1, 0], np.int32)), 998, 3)
    S = Server(gpu)
    gid = S.add(two)
    hit = 0
    for seed in range(1, 6):
        r = S.submit(gid, gpu.Q_BC_SAMPLED, 1, seed)
        if np.diff(two.row)[S.sources(r)[0]] == 0:
            st = C.c_int32()
            S.g.check(S.L.gbc_server_poll(S.h, r, C.byref(st)))
            assert st.value == gpu.REQ_DONE
            hit += 1
        assert S.wait(r) == gpu.REQ_DONE
        st, bc, _, _ = S.fetch(r, gid)
        assert st == 0 and not bc.any()
    assert hit > 0
    assert S.counters()["batches"] == 5 - hit
    S.close()


def test_requests_share_a_lane_group(gpu, orc):
    """On a small-world graph (128-lane groups) requests take 32-lane parts
    of a group: eight 32-source requests need two 128-lane batches (eight if
    each took a whole group), and each result equals a graph handle's
    betweenness over that request's own sources."""
    g = gpu.gen_ba(3000, 4, 12)
    S = Server(gpu, max_lanes=128, workers=1)
    gid = S.add(g)
    rids = [S.submit(gid, gpu.Q_BC_SAMPLED, 32, 900 + i) for i in range(8)]
    for r in rids:
        assert S.wait(r) == gpu.REQ_DONE
    c = S.counters()
    assert c["batches"] <= 4, c
    srcs = [S.sources(r) for r in rids]
    res = [S.fetch(r, gid) for r in rids]
    S.close()
    with gpu.Graph(g) as h:
        for src, (st, bc, _, _) in zip(srcs, res):
            assert st == 0 and len(src) == 32
            assert relerr(bc, h.bc(src)) < TOL
    ref, _ = orc.bc(orc.Graph(g.row, g.col), srcs[3], nthreads=8)
    assert relerr(res[3][1], ref) < TOL


def test_deep_graph_serving_one_lane(gpu, orc):
    """A deep grid of low degree runs one lane per task by default, on a graph
    handle and on the server: requests that share a batch there (32-lane
    parts of one-lane engines) each equal the oracle over their own sources."""
    g = gpu.gen_grid(60, 60, 0.05, seed=7)
    og = orc.Graph(g.row, g.col)
    with gpu.Graph(g) as h:
        src = np.arange(0, g.n, 37, dtype=np.int32)
        bc = h.bc(src)
        assert h.stats()["group_lanes"] == 1
    # path counts on this grid pass 2^64: the oracle's level-scaled FP64 form is the reference
    ref, _ = orc.bc(og, src, scaled=True, nthreads=8)
    assert relerr(bc, ref) < TOL
    S = Server(gpu, max_lanes=256)
    gid = S.add(g)
    rids = [S.submit(gid, gpu.Q_BC_SAMPLED, 40 + 10 * i, 70 + i) for i in range(5)]
    rcc = S.submit(gid, gpu.Q_CC)
    for r in rids + [rcc]:
        assert S.wait(r) == gpu.REQ_DONE
    srcs = [S.sources(r) for r in rids]
    res = [S.fetch(r, gid) for r in rids]
    st, _, cc, _ = S.fetch(rcc, gid)
    c = S.counters()
    S.close()
    assert st == 0 and np.array_equal(cc, orc.cc(og, np.arange(g.n)))
    assert c["shared"] > 0
    for s, (st, b, _, _) in zip(srcs, res):
        ref, _ = orc.bc(og, s, scaled=True, nthreads=8)
        assert st == 0 and relerr(b, ref) < TOL

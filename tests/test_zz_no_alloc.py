"""gbc_cc_noalloc: closeness sums for callers that cannot allocate device
memory at call time (a process that reserved all of HBM for its own pool, a
latency-critical path that must not risk the device synchronisation of
cudaMalloc/cudaFree).  The entry point keeps its BFS state in a fixed
file-scope device array instead of allocating; its results must equal the
allocating entry point gbc_cc exactly, call after call, since every call
reuses (and must re-initialise) the same array.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MAX_VERTICES = 1 << 21


def _noalloc(gpu):
    L = gpu.lib()
    fn = L.gbc_cc_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def test_cc_noalloc_equals_gbc_cc_on_consecutive_calls(gpu):
    torch = pytest.importorskip("torch")
    fn = _noalloc(gpu)
    cases = [(gpu.gen_rmat(13, 8, seed=3), 7), (gpu.gen_er(5000, 2.0, seed=9), 11)]   # 2nd is disconnected
    stream = torch.cuda.current_stream()
    for call, (csr, seed) in enumerate(cases):
        rng = np.random.default_rng(seed)
        src = rng.integers(0, csr.n, 40).astype(np.int32)
        with gpu.Graph(csr) as G:
            ref = G.cc(src)                       # the allocating entry point
        d_row = torch.from_numpy(csr.row).cuda()
        d_col = torch.from_numpy(csr.col).cuda()
        d_src = torch.from_numpy(src).cuda()
        d_out = torch.full((len(src),), -1, dtype=torch.int64, device="cuda")
        st = fn(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), csr.n, C.c_void_p(d_src.data_ptr()),
                len(src), C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert st == 0, gpu.lib().gbc_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy(), ref), f"call {call}"
    # graphs above the fixed scratch size are refused before any device work
    st = fn(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), MAX_VERTICES + 1,
            C.c_void_p(d_src.data_ptr()), 1, C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == 1 and b"scratch" in gpu.lib().gbc_last_error()


def test_cc_noalloc_refuses_a_bad_csr(gpu):
    """A CSR the caller got wrong (an entry equal to n, or a row offset that
    decreases) is refused with GBC_ERR_ARG by the device check that runs
    before the BFS writes anything; a good call right after still equals
    gbc_cc."""
    torch = pytest.importorskip("torch")
    fn = _noalloc(gpu)
    csr = gpu.gen_er(3000, 4.0, seed=5)
    stream = torch.cuda.current_stream()
    src = np.arange(0, csr.n, 97, dtype=np.int32)
    d_src = torch.from_numpy(src).cuda()
    d_out = torch.full((len(src),), -1, dtype=torch.int64, device="cuda")

    def call(row, col):
        d_row = torch.from_numpy(row).cuda()
        d_col = torch.from_numpy(col).cuda()
        st = fn(C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), csr.n, C.c_void_p(d_src.data_ptr()),
                len(src), C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        return st, gpu.lib().gbc_last_error()

    col = csr.col.copy()
    col[len(col) // 2] = csr.n                     # one entry past the last vertex
    st, msg = call(csr.row, col)
    assert st == 1 and b"outside" in msg, msg
    row = csr.row.copy()
    v = int(np.argmax(np.diff(row) > 0)) + 1        # a vertex after one with neighbours
    row[v] = row[v + 1] + 1                         # row[v] > row[v+1]
    st, msg = call(row, csr.col)
    assert st == 1 and b"decrease" in msg, msg
    st, msg = call(csr.row, csr.col)
    assert st == 0, msg
    with gpu.Graph(csr) as G:
        ref = G.cc(src)
    assert np.array_equal(d_out.cpu().numpy(), ref)

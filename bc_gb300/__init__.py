"""bc_gb300 -- Python access to libgbc, the GB300 (sm_103a) betweenness /
closeness library, through its C ABI (include/gbc.h) via ctypes.

The library is built in-tree (``bc_gb300/libgbc.so``, see build.py).  There is
no fallback: if the shared library is missing or a device call fails, the
call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbc.so")

BC_BRANDES, BC_REFERENCE = 0, 1
DELTA_F32, DELTA_F64 = 0, 1
SIGMA_AUTO, SIGMA_EXACT, SIGMA_WIDE = 0, 1, 2
ENGINE_AUTO, ENGINE_PLAIN, ENGINE_LANES = 0, 1, 2
Q_CC, Q_BC, Q_BC_SAMPLED = 0, 1, 2
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = range(5)

STATUS = {0: "GBC_OK", 1: "GBC_ERR_ARG", 2: "GBC_ERR_CUDA", 3: "GBC_ERR_NOMEM", 4: "GBC_ERR_OVERFLOW",
          5: "GBC_ERR_LIMIT", 6: "GBC_ERR_NOT_FOUND", 7: "GBC_ERR_BUSY", 8: "GBC_ERR_TIMEOUT", 9: "GBC_ERR_NO_DEVICE"}


class GbcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Options(C.Structure):
    _fields_ = [("semantics", C.c_int32), ("delta_precision", C.c_int32), ("sigma_mode", C.c_int32),
                ("engine", C.c_int32), ("lanes", C.c_int32), ("sparse_lanes", C.c_int32),
                ("levels_per_graph", C.c_int32), ("source_order", C.c_int32), ("light_steps", C.c_int32),
                ("group_lanes", C.c_int32), ("direction", C.c_int32), ("block_threads", C.c_int32),
                ("bu_share", C.c_int32), ("reserved", C.c_int32 * 3)]


class RunStats(C.Structure):
    _fields_ = [("sources", C.c_int64), ("batches", C.c_int64), ("levels", C.c_int64),
                ("kernel_launches", C.c_int64), ("graph_launches", C.c_int64), ("edges_traversed", C.c_int64),
                ("frontier_entries", C.c_int64), ("sigma_overflow_lanes", C.c_int64), ("kernel_ms", C.c_double),
                ("total_ms", C.c_double), ("lanes", C.c_int32), ("sigma_mode_used", C.c_int32),
                ("fwd_ms", C.c_double), ("bwd_ms", C.c_double), ("fwd_kernels", C.c_int64),
                ("bwd_kernels", C.c_int64), ("group_lanes", C.c_int32), ("bottom_up_levels", C.c_int32),
                ("sigma_bytes", C.c_int32), ("neighbour_visits", C.c_int64)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_ if f[0] != "reserved"}


class ReducedInfo(C.Structure):
    _fields_ = [("n", C.c_int32), ("d1_folded", C.c_int32), ("d1_hubs", C.c_int32), ("alive", C.c_int32),
                ("articulation_points", C.c_int32), ("blocks", C.c_int32), ("max_block", C.c_int32),
                ("block_slots", C.c_int32), ("block_edges", C.c_int64), ("components", C.c_int32),
                ("on_device", C.c_int32), ("fold_rounds", C.c_int32), ("forest_levels", C.c_int32),
                ("reserved", C.c_int32 * 4)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_ if f[0] != "reserved"}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_lanes", C.c_int32), ("max_inflight", C.c_int32),
                ("workers", C.c_int32), ("reserved", C.c_int32 * 7)]


_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_st = C.c_int

# (name, restype, argtypes) of every C-ABI entry point used from Python.
_PROTOS = [
    ("gbc_options_default", None, [C.POINTER(Options)]),
    ("gbc_last_error", C.c_char_p, []),
    ("gbc_version", C.c_char_p, []),
    ("gbc_device_count", C.c_int, []),
    ("gbc_release_cached_memory", _st, []),
    ("gbc_autotune", _st, [_vp, _vp, C.c_int32, C.POINTER(Options), C.POINTER(Options)]),
    ("gbc_graph_create", _st, [_i64p, _i32p, C.c_int32, C.POINTER(_vp)]),
    ("gbc_graph_create_device", _st, [_vp, _vp, C.c_int32, C.c_int64, C.POINTER(_vp)]),
    ("gbc_graph_destroy", _st, [_vp]),
    ("gbc_graph_set_weights", _st, [_vp, _vp, _vp]),
    ("gbc_graph_from_edges", _st, [_i32p, _i32p, C.c_int64, C.c_int32, C.POINTER(_vp)]),
    ("gbc_graph_from_edges_device", _st, [_vp, _vp, C.c_int64, C.c_int32, C.POINTER(_vp)]),
    ("gbc_graph_export", _st, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_int32)]),
    ("gbc_graph_info", _st, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_size_t)]),
    ("gbc_graph_last_stats", _st, [_vp, C.POINTER(RunStats)]),
    ("gbc_bc", _st, [_vp, _vp, C.c_int32, C.POINTER(Options), _f64p]),
    ("gbc_bc_device", _st, [_vp, _vp, C.c_int32, C.POINTER(Options), _vp, _vp]),
    ("gbc_cc", _st, [_vp, _vp, C.c_int32, C.POINTER(Options), _i64p]),
    ("gbc_cc_device", _st, [_vp, _vp, C.c_int32, C.POINTER(Options), _vp, _vp]),
    ("gbc_sssp", _st, [_vp, _i32p, C.c_int32, C.POINTER(Options), _vp, _vp, _vp]),
    ("gbc_reduce", _st, [_i64p, _i32p, C.c_int32, C.c_int32, C.POINTER(_vp)]),
    ("gbc_set_device", _st, [C.c_int]),
    ("gbc_reduce_host", _st, [_i64p, _i32p, C.c_int32, C.c_int32, C.POINTER(_vp)]),
    ("gbc_reduce_device", _st, [_vp, _vp, C.c_int32, C.c_int32, C.POINTER(_vp)]),
    ("gbc_reduced_info_get", _st, [_vp, C.POINTER(ReducedInfo)]),
    ("gbc_cc_reduced", _st, [_vp, C.POINTER(Options), _i64p]),
    ("gbc_bc_reduced", _st, [_vp, C.POINTER(Options), _f64p]),
    ("gbc_reduced_destroy", _st, [_vp]),
    ("gbc_reduced_block_graph", _st, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_int32)]),
    ("gbc_reduced_assemble_cc", _st, [_vp, _i64p, _i64p]),
    ("gbc_reduced_core_graph", _st, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                     C.POINTER(C.c_int32)]),
    ("gbc_reduced_assemble_bc", _st, [_vp, _f64p, _f64p]),
    ("gbc_gen_ba", _st, [C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_vp), C.POINTER(_vp)]),
    ("gbc_gen_rmat", _st, [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int32,
                           C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_int32)]),
    ("gbc_gen_grid", _st, [C.c_int32, C.c_int32, C.c_double, C.c_uint64, C.c_int32, C.POINTER(_vp),
                           C.POINTER(_vp), C.POINTER(C.c_int32)]),
    ("gbc_gen_er", _st, [C.c_int32, C.c_double, C.c_uint64, C.POINTER(_vp), C.POINTER(_vp)]),
    ("gbc_add_pendants", _st, [_i64p, _i32p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_vp),
                               C.POINTER(_vp), C.POINTER(C.c_int32)]),
    ("gbc_add_cycles", _st, [_i64p, _i32p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                             C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_int32)]),
    ("gbc_read_edgelist", _st, [C.c_char_p, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32)]),
    ("gbc_write_scores", _st, [C.c_char_p, _f64p, C.c_int32, C.c_int32, C.c_int32]),
    ("gbc_free", None, [_vp]),
    ("gbc_server_create", _st, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    ("gbc_server_destroy", _st, [_vp]),
    ("gbc_server_add_graph", _st, [_vp, _i64p, _i32p, C.c_int32, C.POINTER(C.c_int32)]),
    ("gbc_server_submit", _st, [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(Options), C.c_double,
                                C.POINTER(C.c_int64)]),
    ("gbc_graph_last_levels", _st, [_vp, _vp, C.c_int32, _vp, _vp, C.c_int32, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("gbc_server_request_bytes", _st, [_vp, C.c_int32, C.c_int32, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("gbc_server_poll", _st, [_vp, C.c_int64, C.POINTER(C.c_int32)]),
    ("gbc_server_wait", _st, [_vp, C.c_int64, C.c_double, C.POINTER(C.c_int32)]),
    ("gbc_server_fetch", _st, [_vp, C.c_int64, _vp, _vp, C.POINTER(C.c_double)]),
    ("gbc_server_cancel", _st, [_vp, C.c_int64]),
    ("gbc_server_sources", _st, [_vp, C.c_int64, _vp, C.c_int32, C.POINTER(C.c_int32)]),
    ("gbc_server_counters", _st, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
]

_LIB = None


def lib():
    """Load libgbc.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m bc_gb300.build` "
                               "(or __graft_entry__.build()); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, res, args in _PROTOS:
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int):
    if status != 0:
        raise GbcError(status, lib().gbc_last_error().decode(errors="replace"))


def options(**kw) -> Options:
    o = Options()
    lib().gbc_options_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, int(v))
    return o


def write_scores(path: str, values: np.ndarray, start: int, end: int, append: bool = False):
    """values[start..end] in the reference's BC_Score.txt layout."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    if end >= len(v):
        raise ValueError("end past the values")
    check(lib().gbc_write_scores(path.encode(), v, int(start), int(end), int(bool(append))))


def device_count() -> int:
    return int(lib().gbc_device_count())


# --------------------------------------------------------------- graphs ----
class CSR:
    """Host CSR: row[n+1] int64, col int32 (both directions of every edge)."""

    def __init__(self, row, col, start: int = 0):
        self.row = np.ascontiguousarray(row, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.n = int(self.row.shape[0] - 1)
        self.start = int(start)

    @property
    def m(self) -> int:
        return int(self.row[-1])


def _take_csr(rp, cp, n, start=0) -> CSR:
    L = lib()
    row = np.ctypeslib.as_array(C.cast(rp, C.POINTER(C.c_int64)), shape=(n + 1,)).copy()
    m = int(row[-1])
    col = np.ctypeslib.as_array(C.cast(cp, C.POINTER(C.c_int32)), shape=(max(m, 1),))[:m].copy()
    L.gbc_free(rp)
    L.gbc_free(cp)
    return CSR(row, col, start)


def gen_ba(n: int, m: int, seed: int) -> CSR:
    rp, cp = _vp(), _vp()
    check(lib().gbc_gen_ba(n, m, seed, C.byref(rp), C.byref(cp)))
    return _take_csr(rp, cp, n)


def gen_rmat(scale: int, edge_factor: int, a=0.57, b=0.19, c=0.19, seed=1, permute=True) -> CSR:
    rp, cp, n = _vp(), _vp(), C.c_int32()
    check(lib().gbc_gen_rmat(scale, edge_factor, a, b, c, seed, int(permute), C.byref(rp), C.byref(cp), C.byref(n)))
    return _take_csr(rp, cp, n.value)


def gen_grid(rows: int, cols: int, remove_frac=0.0, seed=3, largest_only=True) -> CSR:
    rp, cp, n = _vp(), _vp(), C.c_int32()
    check(lib().gbc_gen_grid(rows, cols, remove_frac, seed, int(largest_only), C.byref(rp), C.byref(cp), C.byref(n)))
    return _take_csr(rp, cp, n.value)


def gen_er(n: int, avg_degree: float, seed: int) -> CSR:
    rp, cp = _vp(), _vp()
    check(lib().gbc_gen_er(n, avg_degree, seed, C.byref(rp), C.byref(cp)))
    return _take_csr(rp, cp, n)


def add_pendants(g: CSR, trees: int, max_depth: int, seed: int) -> CSR:
    rp, cp, n = _vp(), _vp(), C.c_int32()
    check(lib().gbc_add_pendants(g.row, g.col, g.n, trees, max_depth, seed, C.byref(rp), C.byref(cp), C.byref(n)))
    return _take_csr(rp, cp, n.value)


def add_cycles(g: CSR, cycles: int, min_len: int, max_len: int, seed: int) -> CSR:
    """Attach cycles of min_len..max_len vertices through uniformly chosen vertices."""
    rp, cp, n = _vp(), _vp(), C.c_int32()
    check(lib().gbc_add_cycles(g.row, g.col, g.n, cycles, min_len, max_len, seed, C.byref(rp), C.byref(cp),
                               C.byref(n)))
    return _take_csr(rp, cp, n.value)


def read_edgelist(path: str) -> CSR:
    rp, cp, n, st = _vp(), _vp(), C.c_int32(), C.c_int32()
    check(lib().gbc_read_edgelist(path.encode(), C.byref(rp), C.byref(cp), C.byref(n), C.byref(st)))
    return _take_csr(rp, cp, n.value, st.value)


class Graph:
    """A device-resident graph (gbc_graph handle)."""

    def __init__(self, csr: CSR):
        self.csr = csr
        self.n = csr.n
        h = _vp()
        check(lib().gbc_graph_create(csr.row, csr.col, csr.n, C.byref(h)))
        self.h = h

    @classmethod
    def from_edges(cls, u, v, n: int) -> "Graph":
        """Build the CSR on the device from an edge list (gbc_graph_from_edges)."""
        uu = np.ascontiguousarray(u, dtype=np.int32)
        vv = np.ascontiguousarray(v, dtype=np.int32)
        if len(uu) != len(vv):
            raise ValueError("u and v differ in length")
        h = _vp()
        check(lib().gbc_graph_from_edges(uu, vv, len(uu), int(n), C.byref(h)))
        g = cls.__new__(cls)
        g.h = h
        g.n = int(n)
        g.csr = g.export()
        return g

    def set_weights(self, w=None, ff=None):
        """Vertex weights (gbc_graph_set_weights): closeness then sums
        ff[v] + d*w[v], betweenness weighs pairs by w[s]*w[t]; None clears."""
        self._w = None if w is None else np.ascontiguousarray(w, dtype=np.int32)
        self._ff = None if ff is None else np.ascontiguousarray(ff, dtype=np.int64)
        for a in (self._w, self._ff):
            if a is not None and len(a) != self.n:
                raise ValueError("weights must have one entry per vertex")
        check(lib().gbc_graph_set_weights(self.h, None if self._w is None else self._w.ctypes.data_as(_vp),
                                          None if self._ff is None else self._ff.ctypes.data_as(_vp)))

    def export(self) -> CSR:
        """The device CSR, copied to the host."""
        rp, cp, n = _vp(), _vp(), C.c_int32()
        check(lib().gbc_graph_export(self.h, C.byref(rp), C.byref(cp), C.byref(n)))
        return _take_csr(rp, cp, n.value)

    def close(self):
        if getattr(self, "h", None):
            lib().gbc_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _src(self, sources):
        if sources is None:
            return None, 0, None
        s = np.ascontiguousarray(sources, dtype=np.int32)
        return s.ctypes.data_as(_vp), len(s), s

    def bc(self, sources=None, **opt) -> np.ndarray:
        out = np.zeros(self.n, np.float64)
        p, k, keep = self._src(sources)
        check(lib().gbc_bc(self.h, p, k, C.byref(options(**opt)), out))
        return out

    def autotune(self, sources=None, **opt) -> dict:
        """Time candidate expansion settings on these sources; later calls
        that leave them to autotuning use the fastest.  Returns the chosen
        lanes / sparse_lanes / light_steps / levels_per_graph / group_lanes /
        block_threads, and on 128-lane groups the closeness direction
        threshold (bu_share; direction 1 when top-down only was fastest)."""
        p, k, keep = self._src(sources)
        ch = Options()
        check(lib().gbc_autotune(self.h, p, k, C.byref(options(**opt)), C.byref(ch)))
        return {f: getattr(ch, f) for f in ("lanes", "sparse_lanes", "light_steps", "levels_per_graph", "group_lanes",
                                            "block_threads", "bu_share", "direction")}

    def cc(self, sources=None, **opt) -> np.ndarray:
        p, k, keep = self._src(sources)
        out = np.zeros(k if k else self.n, np.int64)
        check(lib().gbc_cc(self.h, p, k, C.byref(options(**opt)), out))
        return out

    def sssp(self, sources, **opt):
        s = np.ascontiguousarray(sources, dtype=np.int32)
        dist = np.empty((len(s), self.n), np.int32)
        sig = np.empty((len(s), self.n), np.uint64)
        ovf = np.empty(len(s), np.uint8)
        check(lib().gbc_sssp(self.h, s, len(s), C.byref(options(**opt)), dist.ctypes.data_as(_vp),
                             sig.ctypes.data_as(_vp), ovf.ctypes.data_as(_vp)))
        return dist, sig, ovf.astype(bool)

    def stats(self) -> dict:
        st = RunStats()
        check(lib().gbc_graph_last_stats(self.h, C.byref(st)))
        return st.as_dict()

    def levels(self) -> dict:
        """Level profile of the last lane batch: frontier entries per BFS
        level and device ms per forward / sweep graph launch."""
        nl, nf, nb = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().gbc_graph_last_levels(self.h, None, 0, None, None, 0, C.byref(nl), C.byref(nf), C.byref(nb)))
        ent = np.zeros(max(nl.value, 1), np.int64)
        cap = max(nf.value, nb.value, 1)
        fw, bw = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
        check(lib().gbc_graph_last_levels(self.h, ent.ctypes.data_as(C.c_void_p), nl.value, fw.ctypes.data_as(C.c_void_p),
                                          bw.ctypes.data_as(C.c_void_p), cap, C.byref(nl), C.byref(nf), C.byref(nb)))
        return {"entries": ent[: nl.value], "fwd_ms": fw[: nf.value], "bwd_ms": bw[: nb.value]}


class Reduced:
    """D1-folded, block-split form of a host CSR (gbc_reduced handle).

    on_host=False folds and splits on the device (gbc_reduce); on_host=True
    runs the same reduction on the host (gbc_reduce_host)."""

    def __init__(self, csr: CSR, on_host: bool = False):
        self.csr = csr
        h = _vp()
        fn = lib().gbc_reduce_host if on_host else lib().gbc_reduce
        check(fn(csr.row, csr.col, csr.n, csr.start, C.byref(h)))
        self.h = h

    def info(self) -> dict:
        i = ReducedInfo()
        check(lib().gbc_reduced_info_get(self.h, C.byref(i)))
        return i.as_dict()

    def cc(self, **opt) -> np.ndarray:
        out = np.zeros(self.csr.n, np.int64)
        check(lib().gbc_cc_reduced(self.h, C.byref(options(**opt)), out))
        return out

    def bc(self, **opt) -> np.ndarray:
        out = np.zeros(self.csr.n, np.float64)
        check(lib().gbc_bc_reduced(self.h, C.byref(options(**opt)), out))
        return out

    def block_graph(self):
        """(CSR over block slots, per-slot clone weights)."""
        rp, cp, wp, ns = _vp(), _vp(), _vp(), C.c_int32()
        check(lib().gbc_reduced_block_graph(self.h, C.byref(rp), C.byref(cp), C.byref(wp), C.byref(ns)))
        w = np.ctypeslib.as_array(C.cast(wp, C.POINTER(C.c_int32)), shape=(max(ns.value, 1),))[: ns.value].copy()
        lib().gbc_free(wp)
        return _take_csr(rp, cp, ns.value), w

    def core_graph(self):
        """(CSR over core ids, reach weights, vertex of each core id)."""
        rp, cp, wp, vp, nc = _vp(), _vp(), _vp(), _vp(), C.c_int32()
        check(lib().gbc_reduced_core_graph(self.h, C.byref(rp), C.byref(cp), C.byref(wp), C.byref(vp), C.byref(nc)))
        n = nc.value
        w = np.ctypeslib.as_array(C.cast(wp, C.POINTER(C.c_int32)), shape=(max(n, 1),))[:n].copy()
        v = np.ctypeslib.as_array(C.cast(vp, C.POINTER(C.c_int32)), shape=(max(n, 1),))[:n].copy()
        lib().gbc_free(wp)
        lib().gbc_free(vp)
        return _take_csr(rp, cp, n), w, v

    def assemble_bc(self, core_bc) -> np.ndarray:
        out = np.zeros(self.csr.n, np.float64)
        check(lib().gbc_reduced_assemble_bc(self.h, np.ascontiguousarray(core_bc, dtype=np.float64), out))
        return out

    def assemble_cc(self, D) -> np.ndarray:
        out = np.zeros(self.csr.n, np.int64)
        check(lib().gbc_reduced_assemble_cc(self.h, np.ascontiguousarray(D, dtype=np.int64), out))
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().gbc_reduced_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

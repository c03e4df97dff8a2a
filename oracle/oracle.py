"""ctypes binding of the CPU oracle (``liboracle.so`` built from gbc_oracle.c)
and of the reference's own sequential code built from source into
``oracle/_ref`` (present only where the reference tree was available).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
BC_BRANDES = 0
BC_REFERENCE = 1

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


def build(ref: bool = False, tree: str = "") -> None:
    """Compile liboracle.so (and, with ref=True, the reference's code from
    the tree at `tree`, or GBC_REFERENCE_TREE when `tree` is empty)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref:
        tree = tree or os.environ.get("GBC_REFERENCE_TREE", "")
        if not tree:
            raise RuntimeError("the reference tree is needed: pass tree= or set GBC_REFERENCE_TREE")
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + tree], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_load_edgelist.argtypes = [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int32), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_sssp.argtypes = [C.c_int32, _i64p, _i32p, C.c_int32, _i32p, _u64p, _u8p, _i32p]
        L.orc_bc.argtypes = [C.c_int32, _i64p, _i32p, _i32p, C.c_int32, C.c_int, C.c_int, C.c_int,
                             _f64p, C.POINTER(C.c_int64)]
        L.orc_cc.argtypes = [C.c_int32, _i64p, _i32p, _i32p, C.c_int32, C.c_void_p, C.c_void_p,
                             C.c_int, _i64p]
        L.orc_cc_shared.argtypes = [C.c_int32, _i64p, _i32p, _i32p, C.c_int32, _i64p]
        L.orc_cc_shared.restype = C.c_int64
        L.orc_d1_fold.argtypes = [C.c_int32, _i64p, _i32p, C.c_int32, _i64p, _i64p, _i32p, _i64p,
                                  _i32p, _i32p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.orc_d1_cc.argtypes = [C.c_int32, _i64p, _i32p, C.c_int32, C.c_int, _i64p]
        L.orc_articulation_points.argtypes = [C.c_int32, _i64p, _i32p, C.c_int32, _u8p]
        L.orc_articulation_points.restype = C.c_int32
        L.orc_ap_cc.argtypes = [C.c_int32, _i64p, _i32p, C.c_int32, _i64p]
        L.orc_ap_cc.restype = C.c_int32
        L.orc_components.argtypes = [C.c_int32, _i64p, _i32p, _i32p, C.c_void_p]
        L.orc_components.restype = C.c_int32
        L.orc_gen_rmat.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int,
                                   C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        _LIB = L
    return _LIB


class Graph:
    """CSR over N vertex slots (slot 0 is a phantom vertex for 1-based lists)."""

    def __init__(self, row, col, start=0):
        self.row = np.ascontiguousarray(row, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.N = int(self.row.shape[0] - 1)
        self.start = int(start)

    @property
    def M(self):
        return int(self.row[-1])


def load_edgelist(path: str) -> Graph:
    L = lib()
    N = C.c_int32()
    M = C.c_int64()
    st = C.c_int32()
    rp = C.c_void_p()
    cp = C.c_void_p()
    rc = L.orc_load_edgelist(path.encode(), C.byref(N), C.byref(M), C.byref(st), C.byref(rp), C.byref(cp))
    if rc != 0:
        raise IOError(f"orc_load_edgelist({path}) failed: {rc}")
    row = np.ctypeslib.as_array(C.cast(rp, C.POINTER(C.c_int64)), shape=(N.value + 1,)).copy()
    col = np.ctypeslib.as_array(C.cast(cp, C.POINTER(C.c_int32)), shape=(max(M.value, 1),))[: M.value].copy()
    L.orc_free(rp)
    L.orc_free(cp)
    return Graph(row, col, st.value)


def gen_rmat(scale: int, edge_factor: int, a=0.57, b=0.19, c=0.19, seed=1, permute=True, nthreads=0) -> Graph:
    """Seeded R-MAT graph, the same arrays as the product's generator
    (bc_gb300.gen_rmat) for the same arguments, built without it."""
    L = lib()
    n = C.c_int32()
    rp, cp = C.c_void_p(), C.c_void_p()
    rc = L.orc_gen_rmat(scale, edge_factor, a, b, c, seed, int(bool(permute)), nthreads or (os.cpu_count() or 1),
                        C.byref(n), C.byref(rp), C.byref(cp))
    if rc != 0:
        raise ValueError(f"orc_gen_rmat failed: {rc}")
    row = np.ctypeslib.as_array(C.cast(rp, C.POINTER(C.c_int64)), shape=(n.value + 1,)).copy()
    m = int(row[-1])
    col = np.ctypeslib.as_array(C.cast(cp, C.POINTER(C.c_int32)), shape=(max(m, 1),))[:m].copy()
    L.orc_free(rp)
    L.orc_free(cp)
    return Graph(row, col)


def sssp(g: Graph, s: int):
    L = lib()
    dist = np.empty(g.N, np.int32)
    sig = np.empty(g.N, np.uint64)
    ovf = np.empty(g.N, np.uint8)
    npred = np.empty(g.N, np.int32)
    if L.orc_sssp(g.N, g.row, g.col, int(s), dist, sig, ovf, npred) != 0:
        raise ValueError("bad source")
    return dist, sig, ovf.astype(bool), npred


def bc(g: Graph, sources, semantics=BC_BRANDES, scaled=False, nthreads=1):
    L = lib()
    src = np.ascontiguousarray(sources, dtype=np.int32)
    out = np.zeros(g.N, np.float64)
    novf = C.c_int64(0)
    if L.orc_bc(g.N, g.row, g.col, src, len(src), int(semantics), int(bool(scaled)), int(nthreads), out,
                C.byref(novf)) != 0:
        raise ValueError("bad sources")
    return out, int(novf.value)


def cc(g: Graph, sources, w=None, ff=None, nthreads=1):
    L = lib()
    src = np.ascontiguousarray(sources, dtype=np.int32)
    out = np.zeros(len(src), np.int64)
    wp = ffp = None
    if w is not None:
        w = np.ascontiguousarray(w, dtype=np.int64)
        ff = np.ascontiguousarray(ff, dtype=np.int64)
        wp, ffp = w.ctypes.data, ff.ctypes.data
    if L.orc_cc(g.N, g.row, g.col, src, len(src), wp, ffp, int(nthreads), out) != 0:
        raise ValueError("bad arguments")
    return out


def cc_shared(g: Graph, order=None):
    L = lib()
    if order is None:
        order = np.arange(g.start, g.N, dtype=np.int32)
    order = np.ascontiguousarray(order, dtype=np.int32)
    out = np.zeros(g.N, np.int64)
    runs = L.orc_cc_shared(g.N, g.row, g.col, order, len(order), out)
    return out, int(runs)


def d1_fold(g: Graph):
    L = lib()
    rep = np.empty(g.N, np.int64)
    ff = np.empty(g.N, np.int64)
    par = np.empty(g.N, np.int32)
    lo = np.empty(g.N, np.int64)
    col2 = np.empty(max(g.M, 1), np.int32)
    order = np.empty(g.N, np.int32)
    nf = C.c_int32()
    nh = C.c_int32()
    L.orc_d1_fold(g.N, g.row, g.col, g.start, rep, ff, par, lo, col2, order, C.byref(nf), C.byref(nh))
    return dict(represent=rep, ff=ff, parent=par, live_lo=lo, col=col2, order=order[: nf.value].copy(),
                n_folded=nf.value, n_hub=nh.value)


def d1_cc(g: Graph, fix_components=True):
    out = np.zeros(g.N, np.int64)
    lib().orc_d1_cc(g.N, g.row, g.col, g.start, int(bool(fix_components)), out)
    return out


def articulation_points(g: Graph):
    is_ap = np.zeros(g.N, np.uint8)
    n = lib().orc_articulation_points(g.N, g.row, g.col, g.start, is_ap)
    return is_ap.astype(bool), int(n)


def ap_cc(g: Graph):
    out = np.full(g.N, -1, np.int64)
    n = lib().orc_ap_cc(g.N, g.row, g.col, g.start, out)
    return out, int(n)


def components(g: Graph):
    comp = np.empty(g.N, np.int32)
    size = np.empty(g.N, np.int32)
    n = lib().orc_components(g.N, g.row, g.col, comp, size.ctypes.data)
    return comp, size, int(n)


# --------------------------------------------------------------------------
# The reference's own code, built from source into oracle/_ref (optional).
_REF = {}


def ref_available() -> bool:
    return all(os.path.exists(os.path.join(HERE, "_ref", f)) for f in ("libref_bc.so", "libref_cc.so"))


def _ref(name):
    if name not in _REF:
        L = C.CDLL(os.path.join(HERE, "_ref", name))
        if name == "libref_bc.so":
            L.ref_bc_file.argtypes = [C.c_char_p, C.c_int, C.c_int, _f32p, C.c_int, C.POINTER(C.c_int)]
            L.ref_bc_shared_file.argtypes = [C.c_char_p, _f32p, C.c_int, C.POINTER(C.c_int)]
        else:
            L.ref_cc_file.argtypes = [C.c_char_p, _i32p, C.c_int, C.POINTER(C.c_int)]
            L.ref_d1ap_cc_file.argtypes = [C.c_char_p, _i32p, C.c_int, C.POINTER(C.c_int), _i32p]
        _REF[name] = L
    return _REF[name]


def ref_bc_file(path: str, s_begin=-1, s_end=-1, cap=1 << 24):
    out = np.zeros(cap, np.float32)
    vs = C.c_int()
    rc = _ref("libref_bc.so").ref_bc_file(path.encode(), s_begin, s_end, out, cap, C.byref(vs))
    if rc != 0:
        raise ValueError("capacity")
    return out[: vs.value - 1].copy()


def ref_bc_shared_file(path: str, cap=1 << 24):
    """The reference's computeBC_shareBased (Seq_Brandes/Brandes.c:374), FP32."""
    out = np.zeros(cap, np.float32)
    vs = C.c_int()
    if _ref("libref_bc.so").ref_bc_shared_file(path.encode(), out, cap, C.byref(vs)) != 0:
        raise ValueError("capacity")
    return out[: vs.value - 1].copy()


def ref_cc_file(path: str, cap=1 << 24):
    out = np.zeros(cap, np.int32)
    vs = C.c_int()
    if _ref("libref_cc.so").ref_cc_file(path.encode(), out, cap, C.byref(vs)) != 0:
        raise ValueError("capacity")
    return out[: vs.value - 1].copy()


def ref_d1ap_cc_file(path: str, cap=1 << 24):
    out = np.zeros(cap, np.int32)
    vs = C.c_int()
    st = np.zeros(8, np.int32)
    if _ref("libref_cc.so").ref_d1ap_cc_file(path.encode(), out, cap, C.byref(vs), st) != 0:
        raise ValueError("capacity")
    return out[: vs.value - 1].copy(), dict(d1=int(st[0]), hub=int(st[1]), ordinary=int(st[2]), ap=int(st[3]),
                                            comp=int(st[4]), max_comp=int(st[5]), end_id=int(st[6]))

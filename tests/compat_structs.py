"""ctypes mirrors of the reference structs declared in include/gbc_compat.h
(field order and types of Lib/CSR/CSR.h:34-95 and Lib/AdjList/AdjList.h)."""
import ctypes as C
import os

P = C.POINTER
I = C.c_int


class QQueue(C.Structure):
    _fields_ = [("dataArr", P(I)), ("front", I), ("rear", I), ("size", I)]


class CSR(C.Structure):
    _fields_ = [
        ("csrV", P(I)), ("csrE", P(I)), ("csrVSize", I), ("csrESize", I), ("csrNodesDegree", P(I)),
        ("oriCsrV", P(I)), ("oriCsrNodesDegree", P(I)), ("nodesType", P(C.c_uint)),
        ("representNode", P(I)), ("ff", P(I)), ("degreeOneNodesQ", P(QQueue)), ("notD1Node", P(I)),
        ("D1Parent", P(I)), ("foldedDegreeOneCount", I), ("hubNodeCount", I), ("ordinaryNodeCount", I),
        ("startAtZero", I), ("maxDegree", I), ("startNodeID", I), ("endNodeID", I), ("totalNodeNumber", I),
        ("low", P(I)), ("depth_level", P(I)), ("Dfs_sequence", P(I)), ("ap_count", I), ("AP_List", P(I)),
        ("AP_component_number", P(I)), ("compID", P(I)), ("apCloneTrackOriAp_ID", P(I)), ("apCloneCount", I),
        ("compNum", I), ("maxCompSize_afterSplit", I), ("aliveNode", P(I)), ("aliveNodeCount", I),
        ("aliveNodeFlags", P(I)), ("comp_NodesID_CsrData", P(I)), ("comp_CsrOffset", P(I)),
        ("nodesCompID", P(I)), ("mapNodeID_New_to_Old", P(I)), ("mapNodeID_Old_to_new", P(I)),
        ("orderedCsrV", P(I)), ("orderedCsrE", P(I)), ("newEndID", I), ("comp_newNodesID_CsrData", P(I)),
        ("comp_newCsrOffset", P(I)), ("newNodesCompID", P(I)), ("compEndID", I), ("BCs", P(C.c_float)),
        ("CCs", P(I)),
    ]


def bind(L):
    L.buildGraph.restype = C.c_void_p
    L.buildGraph.argtypes = [C.c_char_p]
    L.createCSR.restype = P(CSR)
    L.createCSR.argtypes = [C.c_void_p]
    for name in ("computeBC", "computeBC_shareBased"):
        getattr(L, name).argtypes = [P(CSR), P(C.c_float)]
        getattr(L, name).restype = None
    L.computeCC.argtypes = [P(CSR), P(I)]
    L.computeCC.restype = P(I)
    for name in ("computeCC_shareBased", "compute_D1_CC", "compute_D1_AP_CC_shareBased_DegreeOrder"):
        getattr(L, name).argtypes = [P(CSR), P(I)]
        getattr(L, name).restype = None
    for name in ("D1Folding", "AP_detection", "gpu_vb", "preprocess_then_parallel_sharedBased_DegreeOrder"):
        getattr(L, name).argtypes = [P(CSR)]
        getattr(L, name).restype = None
    L.gpu_fan.argtypes = [C.c_void_p, P(CSR)]
    L.gpu_fan.restype = None
    return L


def load(L, path):
    g = L.buildGraph(path.encode())
    return g, L.createCSR(g)


def build_dropin_driver(gbc, out_dir):
    """Compile tests/dropin_driver.c with gcc against include/gbc_compat.h and
    link it with -lgbc, as a reference driver would be; returns the binary."""
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    libdir = os.path.dirname(gbc.build.LIB)
    exe = os.path.join(str(out_dir), "dropin_driver")
    cmd = ["gcc", "-O2", "-Wall", "-I", os.path.join(root, "include"), os.path.join(here, "dropin_driver.c"),
           "-L", libdir, "-lgbc", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe

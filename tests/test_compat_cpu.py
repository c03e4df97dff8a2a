"""The struct-CSR drop-in ingest and reductions, on CPU: layouts follow the
reference's conventions (Lib/CSR/CSR.c:9-108) and the struct-level D1
folding / AP detection reproduce the reference's structural counts."""
import ctypes as C
import json
import os

import numpy as np

from compat_structs import bind, build_dropin_driver, load

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_create_csr_layout(gbc, datasets):
    L = bind(gbc.lib())
    for name in ["karate.txt", "polbooks.txt", "testdata2.txt"]:
        g, c = load(L, datasets[name])
        c = c.contents
        ref = gbc.read_edgelist(datasets[name])
        one_based = ref.start == 1
        assert c.startAtZero == (0 if one_based else 1)
        assert c.csrVSize == ref.n + (1 if True else 0) - 0 or True
        assert c.startNodeID == ref.start and c.endNodeID == ref.n - 1
        assert c.csrVSize == ref.n + 1
        if one_based:
            assert c.csrV[0] == -1
        assert c.csrESize == ref.m
        for v in range(ref.start, ref.n):
            assert c.csrV[v] == ref.row[v] and c.csrV[v + 1] == ref.row[v + 1]
        assert [c.csrE[i] for i in range(ref.m)] == list(ref.col)
        assert c.totalNodeNumber == ref.n - ref.start


def test_struct_reductions_match_reference_counts(gbc, datasets):
    L = bind(gbc.lib())
    struct = json.load(open(os.path.join(GOLDEN, "structure.json")))
    for name, st in struct.items():
        g, c = load(L, datasets[name])
        L.D1Folding(c)
        cc = c.contents
        assert (cc.foldedDegreeOneCount, cc.hubNodeCount, cc.ordinaryNodeCount) == (st["d1"], st["hub"], st["ordinary"])
        L.AP_detection(c)
        assert c.contents.ap_count == st["ap"], name


def test_dropin_driver_compiles_and_links(gbc, tmp_path):
    """A C driver written against include/gbc_compat.h builds with gcc and links
    with -lgbc alone: every symbol of the struct-CSR sequence it calls
    (buildGraph, createCSR, computeBC, computeCC, the D1+AP closeness) is
    exported with a C signature."""
    exe = build_dropin_driver(gbc, tmp_path)
    assert os.path.exists(exe)

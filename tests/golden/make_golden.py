"""Regenerates the golden fixtures under tests/golden/ from the reference tree.

Run where the reference is mounted (its path as argv[1], or in the
environment variable GBC_REFERENCE_TREE), after `make -C oracle ref` built the reference's own
sequential code from its sources into oracle/_ref.  It
  * copies the shipped edge-list datasets used by the tests (gzip'd; these
    are public graph datasets, not code) and the reference's golden BC file
    for karate (reference/karate_BC_Score.txt),
  * records, per dataset, the reference's own outputs: plain closeness sums
    (Seq_CC/CC.cpp:37 computeCC), the D1+AP closeness of the release path
    (Seq_CC/CC.cpp:1728) with its structural counts, the reference's FP32
    betweenness (Seq_Brandes/Brandes.c:224), and -- for the smaller graphs --
    its shared-traversal variant (Seq_Brandes/Brandes.c:374).
The GPU machine has no reference tree; the tests read only these fixtures.
"""
import gzip
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBC_REFERENCE_TREE", "")
DATASETS = ["karate.txt", "dolphins.txt", "football.txt", "polbooks.txt", "testdata.txt", "testdata1.txt",
            "testdata2.txt", "ia-fb-messages.mtx", "tech-WHOIS.mtx", "caida.mtx", "ia-email-EU.mtx", "ca-HepPh.mtx"]
BC_SMALL = {"karate.txt", "dolphins.txt", "football.txt", "polbooks.txt", "testdata.txt", "testdata1.txt",
            "testdata2.txt", "ia-fb-messages.mtx"}


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py <reference tree> (or set GBC_REFERENCE_TREE)")
    O.build(ref=True, tree=REF)
    os.makedirs(os.path.join(HERE, "datasets"), exist_ok=True)
    meta = {}
    for name in DATASETS:
        src = os.path.join(REF, "dataset", name)
        dst = os.path.join(HERE, "datasets", name + ".gz")
        with open(src, "rb") as f, open(dst, "wb") as raw:
            with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                shutil.copyfileobj(f, g)
        cc = O.ref_cc_file(src)
        d1ap, stats = O.ref_d1ap_cc_file(src)
        out = {"cc_ref": cc.astype(np.int64), "d1ap_cc_ref": d1ap.astype(np.int64)}
        out["bc_ref_f32"] = O.ref_bc_file(src)
        if name in BC_SMALL:
            out["bc_shared_ref_f32"] = O.ref_bc_shared_file(src)
        np.savez_compressed(os.path.join(HERE, name.split(".")[0] + ".npz"), **out)
        meta[name] = stats
        print(name, stats, flush=True)
    shutil.copyfile(os.path.join(REF, "karate_BC_Score.txt"), os.path.join(HERE, "karate_BC_Score.txt"))
    with open(os.path.join(HERE, "structure.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()

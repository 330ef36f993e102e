"""Record what the reference's HITTER=1 build gives on every golden input.

DAKC's Makefile builds with HITTER=0 (dakc/Makefile:11), which the golden
tables pin; the header's default is HITTER=1 (dakc/src/common/common.hpp:42-44),
which pre-aggregates each 10,000-k-mer flush buffer and sends k-mers seen
three or more times as (k-mer, count) pairs (kcounter.cpp:146-245, 325-383).
This script runs the reference's counting sources built with -DHITTER=1
(oracle/Makefile `ref H=1`, the same harness and PE counts as
make_golden.py) on each fixture's input and writes tests/golden/hitter1.json:
per case the table's SHA-256 (keys then counts), whether it equals the
HITTER=0 fixture, and, where it does not, the HITTER=1 table itself.
Needs the reference tree; run from the repo root:

    python tests/golden/make_hitter1.py
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402


def digest(keys, counts) -> str:
    return hashlib.sha256(np.ascontiguousarray(keys, np.uint64).tobytes() +
                          np.ascontiguousarray(counts, np.uint32).tobytes()).hexdigest()


def main():
    with open(os.path.join(HERE, "index.json")) as f:
        index = json.load(f)["cases"]
    out = {}
    for path in sorted(glob.glob(os.path.join(HERE, "*.npz"))):
        name = os.path.basename(path)[:-4]
        z = np.load(path)
        W, k = int(z["W"]), int(z["k"])
        runs = {}
        for p in index[name]["pes"]:
            (keys, counts, nk), _ = pyoracle.ref_table(z["text"], W, k, pes=p, hitter=1)
            same = (nk == int(z["n_kmers"]) and np.array_equal(keys, z["keys"])
                    and np.array_equal(counts, z["counts"]))
            ent = {"n_kmers": int(nk), "n_distinct": int(keys.size),
                   "table_sha256": digest(keys, counts), "equals_hitter0": bool(same)}
            if not same:
                ent["keys"] = [int(x) for x in keys]
                ent["counts"] = [int(x) for x in counts]
            runs[str(p)] = ent
            print(name, p, "same" if same else "differs", nk, int(z["n_kmers"]))
        out[name] = runs
    with open(os.path.join(HERE, "hitter1.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_hitter1.py",
                   "reference": "dakc/src/kcounter/{kcounter.cpp,kcounter_funcs.cpp} via oracle/shim, "
                                "HITTER=1 BIGKSIZE=16 KCOUNT_BUCKET_SIZE=10000",
                   "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()

"""Generate the golden (k-mer, count) tables under tests/golden/ by running the
reference's own counting code.

The reference ships no tests, fixtures or known-answer vectors, so its
behaviour is pinned here by running its kcounter sources
(dakc/src/kcounter/kcounter.cpp + kcounter_funcs.cpp, compiled unmodified
against oracle/shim with -DKMERLEN=k -DREADLEN=W -DHITTER=0, the Makefile's
setting) on seeded inputs, and storing the merged table each run produced.
Needs the reference tree (default /root/reference); run from the repo root:

    python tests/golden/make_golden.py

Every case runs the reference with one PE and, where each PE receives k-mers,
with several PEs too (the table must not depend on the PE count).  Each
fixture stores the input text itself, so the checks never depend on a
generator's output staying the same.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dakc_gb300 import synth  # noqa: E402
from oracle import pyoracle  # noqa: E402


def lines(rows, W):
    out = b""
    for r in rows:
        out += r + b"M" * (W - len(r)) + b"\n"
    return np.frombuffer(out, dtype=np.uint8)


def cases():
    edge_rows = [b"ACGTACGTACGTACGTACGT", b"acgtNacgtacgtACGT", b"ACGTACGM", b"ACGTAC\nGTAC",
                 b"AAAAAAAAAAAAAAAAAAAA", b"TTTT TTTT-TTTTTTT", b"CCCCMCCCCCCCCC",
                 b"GATTACAGATTACAGATTAC", b"NNNNNNNNNNNNNNNNNNNA", b"ACGTACGTACGTACGTACNA",
                 b"gggggggggggggggggggg", b"CATMAAAAAAAAAAAAAAAA"]
    edge = lines(edge_rows, 20)
    for k in (1, 2, 3, 5, 13, 20):
        yield f"edge_w20_k{k}", edge, 20, k, (1,)
    nul = lines([b"ACGTACGTAC", b"CCCCCCCCCC", b"\0GGGGGGGGG", b"TTTTTTTTTT"], 10)
    yield "nul_line_w10_k4", nul, 10, 4, (1,)
    rnd = synth.random_lines(7, 400, 150, b"ACGTACGTACGTacgtNM")
    for k in (17, 31):
        yield f"random_w150_k{k}", rnd, 150, k, (1, 4)
    g = synth.genome_uniform(31, 300_000)
    reads = synth.reads(32, g, 500, 150, 150, 150, rc_frac=0.5, err_rate=0.01)
    for k in (17, 21, 31):
        yield f"reads_w150_k{k}", reads, 150, k, (1, 4)
    var = synth.reads(33, g, 400, 100, 250, 250, rc_frac=0.5, err_rate=0.005)
    yield "varlen_w250_k31", var, 250, 31, (1, 3)
    k32 = synth.reads(34, g, 400, 90, 100, 100, rc_frac=0.5, err_rate=0.01)
    yield "reads_w100_k32", k32, 100, 32, (1, 2)
    rep = np.concatenate([np.tile(synth.reads(35, g, 2, 150, 150, 150, rc_frac=0.0), 500),
                          synth.reads(36, g, 200, 150, 150, 150, rc_frac=0.5, err_rate=0.01)])
    yield "skew_w150_k31", rep, 150, 31, (1, 4)


def main():
    index = {}
    for name, text, W, k, pes in cases():
        tables = []
        for p in pes:
            (keys, counts, nk), _ = pyoracle.ref_table(text, W, k, pes=p)
            tables.append((keys, counts, nk))
        for t in tables[1:]:
            assert np.array_equal(t[0], tables[0][0]) and np.array_equal(t[1], tables[0][1]), name
        keys, counts, nk = tables[0]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), text=text, W=W, k=k, keys=keys,
                            counts=counts, n_kmers=nk)
        index[name] = {"W": W, "k": k, "pes": list(pes), "n_distinct": int(keys.size),
                       "n_kmers": int(nk), "text_sha256": hashlib.sha256(text.tobytes()).hexdigest()}
        print(name, keys.size, nk)
    # the 1 Mbp plain workload: too large to store, so its table is pinned by a digest
    rs = synth.plain_1m()
    (keys, counts, nk), _ = pyoracle.ref_table(rs.text, 150, 31, pes=8)
    h = hashlib.sha256(keys.tobytes() + counts.tobytes()).hexdigest()
    index["plain_1m"] = {"W": 150, "k": 31, "pes": [8], "n_distinct": int(keys.size),
                         "n_kmers": int(nk), "table_sha256": h,
                         "text_sha256": hashlib.sha256(rs.text.tobytes()).hexdigest()}
    print("plain_1m", keys.size, nk, h)
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_golden.py",
                   "reference": "dakc/src/kcounter/{kcounter.cpp,kcounter_funcs.cpp} via oracle/shim, "
                                "HITTER=0 BIGKSIZE=16 KCOUNT_BUCKET_SIZE=10000",
                   "cases": index}, f, indent=1)


if __name__ == "__main__":
    main()

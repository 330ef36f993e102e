"""Time the C port of DAKC's two phases against the reference's own counting
code at the same PE count, on the same reads (test infrastructure).

The reference side is oracle/_ref (dakc/src/kcounter/kcounter.cpp and
kcounter_funcs.cpp compiled unmodified against oracle/shim, one forked process
per PE); its time is the "kmer counting time" DAKC prints itself
(kcounter.cpp:262, 416-430: phase 1 + phase 2, max over PEs).  The port's
time is dko_dakc_port's phase 1 + phase 2 on P threads.  Both tables are
checked equal.  Needs the reference tree (to build oracle/_ref):

    python oracle/calibrate.py [--pes P] [--reads N] [--runs R]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from dakc_gb300 import synth  # noqa: E402
from oracle import pyoracle  # noqa: E402


def ref_seconds(out: str) -> float:
    m = re.search(r"kmer counting time: ([0-9.eE+-]+) seconds", out)
    if not m:
        raise RuntimeError("no timing line in the reference's output")
    return float(m.group(1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pes", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--reads", type=int, default=2_000_000,
                    help="reads of the large_100m workload (its first N)")
    args = ap.parse_args()
    rows = []
    large = synth.large_100m()
    cases = [("plain_1m", synth.plain_1m().text),
             (f"large_100m first {args.reads:,} reads", large.text[: args.reads * 151])]
    for name, text in cases:
        ref_t, port_t = [], []
        for _ in range(args.runs):
            (rk, rc, rn), out = pyoracle.ref_table(text, 150, 31, pes=args.pes)
            ref_t.append(ref_seconds(out))
            (pk, pc, pn), secs = pyoracle.dakc_port(text, 150, 31, args.pes, merge=True)
            port_t.append(secs)
            assert rn == pn and np.array_equal(rk, pk) and np.array_equal(rc, pc)
        row = {"input": name, "kmers": int(rn), "pes": args.pes,
               "reference_s": float(np.median(ref_t)), "port_s": float(np.median(port_t))}
        row["port_over_reference_speed"] = row["reference_s"] / row["port_s"]
        rows.append(row)
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()

"""Generate the golden fixtures of the read-format rows by running the
reference's own code: syngen/fq2txtmaker.sh and syngen/fq2famaker.sh
(bash/awk/sed, run where they lie on a FASTQ written here), DAKC's counting
sources on the converted text (oracle/_ref, as make_golden.py does), and
PakMan*'s k-mer counting (pakman_star/src/kmer_counting.cpp compiled
unmodified against the one-rank MPI stand-in, oracle/_ref/pakman_ref_k<k>)
on the converted FASTA.  Needs the reference tree; run from the repo root:

    python tests/golden/make_formats.py

Writes tests/golden/formats/formats_*.npz (each holds its inputs and outputs)
and tests/golden/formats/formats.json (SHA-256 digests).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402

SYNGEN = os.path.join(pyoracle.REFERENCE_TREE, "syngen")


def var_reads(seed, n, lo, hi):
    """Reads of uneven length from a random genome, some lower case, some
    with N, one with a space (fq2txtmaker.sh turns every space into 'M')."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = rng.choice(np.frombuffer(b"ACGT", np.uint8), 50_000)
    out = []
    for i in range(n):
        L = int(rng.integers(lo, hi + 1))
        s = int(rng.integers(0, g.size - L))
        r = g[s:s + L].copy()
        if i % 7 == 0:
            r[rng.integers(0, L)] = ord("N")
        if i % 11 == 0:
            r[: L // 3] |= 0x20
        if i == 5:
            r[L // 2] = ord(" ")
        out.append(r.tobytes())
    return out


def fastq(reads):
    return b"".join(b"@r%d\n%s\n+\n%s\n" % (i, r, b"I" * len(r)) for i, r in enumerate(reads))


def run_script(script: str, fq: bytes, ext: str) -> bytes:
    """Run a syngen conversion script on one .fq in a scratch directory."""
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "reads.fq"), "wb") as f:
            f.write(fq)
        subprocess.run(["bash", os.path.join(SYNGEN, script)], cwd=d, check=True)
        with open(os.path.join(d, "reads" + ext), "rb") as f:
            return f.read()


def sha(*arrs) -> str:
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    if not shutil.which("awk") or not shutil.which("sed"):
        raise SystemExit("awk and sed are needed")
    index = {}
    for name, seed, n, lo, hi in (("formats_mixed", 21, 400, 60, 150),
                                  ("formats_long", 22, 200, 150, 250)):
        reads = var_reads(seed, n, lo, hi)
        fq = fastq(reads)
        txt = run_script("fq2txtmaker.sh", fq, ".txt")
        fa = run_script("fq2famaker.sh", fq, ".fa")
        w = len(txt.split(b"\n", 1)[0])
        entry = {"reads": n, "line_width": w, "fastq_sha256": hashlib.sha256(fq).hexdigest(),
                 "txt_sha256": hashlib.sha256(txt).hexdigest(),
                 "fa_sha256": hashlib.sha256(fa).hexdigest()}
        arrays = {"fastq": np.frombuffer(fq, np.uint8), "txt": np.frombuffer(txt, np.uint8),
                  "fa": np.frombuffer(fa, np.uint8), "W": w}
        for k in (21, 31):
            (dk_k, dk_c, nk), _ = pyoracle.ref_table(np.frombuffer(txt, np.uint8), w, k, pes=1)
            pk_k, pk_c = pyoracle.pakman_ref_table(fa, k)
            pk_k2, pk_c2 = pyoracle.pakman_ref_table(fa, k, batch=997)  # several transfers
            assert np.array_equal(pk_k, pk_k2) and np.array_equal(pk_c, pk_c2)
            arrays.update({f"dakc_keys_k{k}": dk_k, f"dakc_counts_k{k}": dk_c,
                           f"dakc_nk_k{k}": nk,
                           f"pakman_keys_k{k}": pk_k, f"pakman_counts_k{k}": pk_c})
            entry[f"dakc_k{k}"] = {"n_distinct": int(dk_k.size), "n_kmers": int(nk),
                                   "table_sha256": sha(dk_k, dk_c)}
            entry[f"pakman_k{k}"] = {"n_distinct": int(pk_k.size),
                                     "n_kmers": int(pk_c.astype(np.uint64).sum()),
                                     "table_sha256": sha(pk_k, pk_c)}
        np.savez_compressed(os.path.join(HERE, "formats", f"{name}.npz"), **arrays)
        index[name] = entry
        print(name, w, entry["dakc_k31"], entry["pakman_k31"])
    with open(os.path.join(HERE, "formats", "formats.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_formats.py",
                   "reference": "syngen/fq2txtmaker.sh, syngen/fq2famaker.sh; "
                                "dakc/src/kcounter via oracle/shim (HITTER=0); "
                                "pakman_star/src/kmer_counting.cpp via oracle/shim_pakman "
                                "(LMER_LENGTH=8, FAST, one rank)",
                   "cases": index}, f, indent=1)


if __name__ == "__main__":
    main()

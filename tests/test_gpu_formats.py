"""Reads in other layouts (dk_count_format) and the PakMan* convention: exact
against the oracle's restatements of the reference's conversion
(fq2txtmaker.sh) + DAKC's count, and of PakMan*'s FASTA walk."""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def var_reads(seed, n, lo=60, hi=250):
    """Reads of uneven length from a random genome, some lower case, some N."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = rng.choice(np.frombuffer(b"ACGT", np.uint8), 200_000)
    out = []
    for i in range(n):
        L = int(rng.integers(lo, hi + 1))
        s = int(rng.integers(0, g.size - L))
        r = g[s:s + L].copy()
        if i % 7 == 0:
            r[rng.integers(0, L)] = ord("N")
        if i % 11 == 0:
            r[: L // 3] |= 0x20
        out.append(r.tobytes())
    return out


def fastq(reads):
    return b"".join(b"@r%d\n%s\n+\n%s\n" % (i, r, b"I" * len(r)) for i, r in enumerate(reads))


def fasta(reads, lead=b""):
    return lead + b"".join(b">r%d\n%s\n" % (i, r) for i, r in enumerate(reads))


@pytest.mark.parametrize("k", [17, 31])
def test_fastq_matches_fq2txt_then_dakc(engine, k):
    reads = var_reads(1, 3000)
    reads[5] = reads[5][:40] + b" " + reads[5][41:]        # a space becomes 'M' (fq2txtmaker)
    fq = fastq(reads)
    txt, w = pyoracle.fq2txt(fq)
    keys, counts, nk = pyoracle.count(np.frombuffer(txt, np.uint8), w, k)
    r, width = engine.count_format(fq, dk.FORMAT_FASTQ, k, dk.CONV_DAKC)
    assert width == w
    assert r.n_kmers == nk and np.array_equal(r.kmers, keys) and np.array_equal(r.counts, counts)
    # an explicit, wider line width gives the same table
    r2, w2 = engine.count_format(fq, dk.FORMAT_FASTQ, k, dk.CONV_DAKC, line_width=w + 9)
    assert w2 == w + 9 and np.array_equal(r2.kmers, keys) and np.array_equal(r2.counts, counts)


@pytest.mark.parametrize("k", [13, 21, 31])
def test_fasta_pakman_convention(engine, k):
    reads = var_reads(2, 2500)
    fa = fasta(reads, lead=b"; a comment line before the first record\n")
    keys, counts, nk = pyoracle.table_of(pyoracle.pakman_kmers(fa, k))
    for variant in (dk.VARIANT_HASH, dk.VARIANT_SORT):
        r, width = engine.count_format(fa, dk.FORMAT_FASTA, k, dk.CONV_PAKMAN, variant=variant)
        assert width == max(len(x) for x in reads)
        assert r.n_kmers == nk and np.array_equal(r.kmers, keys), variant
        assert np.array_equal(r.counts, counts), variant
    # no final newline
    keys2, counts2, nk2 = pyoracle.table_of(pyoracle.pakman_kmers(fa[:-1], k))
    r, _ = engine.count_format(fa[:-1], dk.FORMAT_FASTA, k, dk.CONV_PAKMAN)
    assert r.n_kmers == nk2 and np.array_equal(r.kmers, keys2) and np.array_equal(r.counts, counts2)


def test_plain_lines_both_conventions(engine):
    reads = var_reads(3, 2000, 20, 180)
    text = b"\n".join(reads) + b"\n"
    k = 21
    keys, counts, nk = pyoracle.table_of(pyoracle.pakman_kmers(b">\n" + b"\n>\n".join(reads) + b"\n", k))
    r, _ = engine.count_format(text, dk.FORMAT_LINES, k, dk.CONV_PAKMAN)
    assert r.n_kmers == nk and np.array_equal(r.kmers, keys) and np.array_equal(r.counts, counts)
    w = max(len(x) for x in reads)
    padded = b"".join(x.ljust(w, b"M") + b"\n" for x in reads)
    keys, counts, nk = pyoracle.count(np.frombuffer(padded, np.uint8), w, k)
    r, width = engine.count_format(text, dk.FORMAT_LINES, k, dk.CONV_DAKC)
    assert width == w and r.n_kmers == nk and np.array_equal(r.kmers, keys)


def test_format_edge_cases(engine):
    r, _ = engine.count_format(b"", dk.FORMAT_FASTQ, 21)
    assert r.n_kmers == 0 and r.kmers.size == 0
    r, _ = engine.count_format(b"no record marker here\nACGTACGT\n", dk.FORMAT_FASTA, 3, dk.CONV_PAKMAN)
    assert r.n_kmers == 0
    with pytest.raises(dk.DkError):       # a read longer than the line width asked for
        engine.count_format(b"ACGTACGTAC\n", dk.FORMAT_LINES, 3, dk.CONV_DAKC, line_width=5)
    with pytest.raises(dk.DkError):       # reads of more than 1,024 bytes
        engine.count_format(b">h\n" + b"A" * 1100 + b"\n", dk.FORMAT_FASTA, 3, dk.CONV_PAKMAN)


@pytest.mark.parametrize("k", [11, 25, 32])
def test_fasta_pakman_long_reads(engine, k):
    """Reads of 257-1,024 bytes under PakMan*'s convention take the
    warp-per-line kernels: exact against the oracle's restatement of
    PakMan*'s FASTA walk, both variants."""
    reads = var_reads(7, 600, lo=257, hi=1024)
    fa = fasta(reads)
    keys, counts, nk = pyoracle.table_of(pyoracle.pakman_kmers(fa, k))
    for variant in (dk.VARIANT_HASH, dk.VARIANT_SORT):
        if k == 32 and variant == dk.VARIANT_HASH:
            continue  # k = 32 always sorts
        r, width = engine.count_format(fa, dk.FORMAT_FASTA, k, dk.CONV_PAKMAN, variant=variant)
        assert width == max(len(x) for x in reads)
        assert r.n_kmers == nk and np.array_equal(r.kmers, keys) and np.array_equal(r.counts, counts)


def test_pakman_long_fixed_lines(engine):
    """dk_count on fixed-width lines of 700 bytes under PakMan*'s
    convention: reads shorter than the width end at their '\\n' padding."""
    reads = var_reads(8, 400, lo=100, hi=700)
    text = b"".join(x + b"\n" * (700 - len(x)) + b"\n" for x in reads)
    keys, counts, nk = pyoracle.table_of(pyoracle.pakman_kmers(fasta(reads), 21))
    d = dk.Engine.desc(700, 21, dk.VARIANT_HASH)
    d.convention = dk.CONV_PAKMAN
    buf = np.frombuffer(text, np.uint8)
    t = engine.count_raw(buf.ctypes.data, buf.size, d)
    try:
        n = int(t.n)
        got_k = np.ctypeslib.as_array(t.kmers, shape=(n,)).copy()
        got_c = np.ctypeslib.as_array(t.counts, shape=(n,)).copy()
        assert int(t.n_kmers) == nk
    finally:
        engine.free_table(t)
    assert np.array_equal(got_k, keys) and np.array_equal(got_c, counts)


import glob  # noqa: E402
import os  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FORMAT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "formats", "formats_*.npz")))


@pytest.mark.parametrize("path", FORMAT_FIXTURES, ids=[os.path.basename(p)[:-4] for p in FORMAT_FIXTURES])
@pytest.mark.parametrize("k", [21, 31])
def test_formats_match_reference_runs(engine, path, k):
    """FASTQ through dk_count_format equals DAKC's table of fq2txtmaker.sh's
    text, and the same reads as FASTA (fq2famaker.sh) under the PakMan*
    convention equal PakMan*'s own table -- both produced by running the
    reference's code (tests/golden/make_formats.py)."""
    z = np.load(path)
    r, width = engine.count_format(z["fastq"].tobytes(), dk.FORMAT_FASTQ, k, dk.CONV_DAKC)
    assert width == int(z["W"])
    assert r.n_kmers == int(z[f"dakc_nk_k{k}"])
    assert np.array_equal(r.kmers, z[f"dakc_keys_k{k}"])
    assert np.array_equal(r.counts, z[f"dakc_counts_k{k}"])
    for variant in (dk.VARIANT_HASH, dk.VARIANT_SORT):
        r, _ = engine.count_format(z["fa"].tobytes(), dk.FORMAT_FASTA, k, dk.CONV_PAKMAN,
                                   variant=variant)
        assert np.array_equal(r.kmers, z[f"pakman_keys_k{k}"]), variant
        assert np.array_equal(r.counts, z[f"pakman_counts_k{k}"]), variant

"""The CPU oracle, pinned against the reference's own output (CPU only).

tests/golden/*.npz hold tables produced by the reference's counting sources
(see tests/golden/make_golden.py).  The oracle must reproduce every one bit
for bit before it is trusted as the GPU engine's checker.
"""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

from dakc_gb300 import synth
from oracle import pyoracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(path):
    z = np.load(path)
    return z["text"], int(z["W"]), int(z["k"]), z["keys"], z["counts"], int(z["n_kmers"])


def test_fixtures_present():
    assert len(FIXTURES) >= 10
    with open(os.path.join(GOLDEN, "index.json")) as f:
        idx = json.load(f)["cases"]
    for p in FIXTURES:
        name = os.path.basename(p)[:-4]
        text, W, k, keys, counts, nk = load(p)
        assert idx[name]["text_sha256"] == hashlib.sha256(text.tobytes()).hexdigest()
        assert idx[name]["n_distinct"] == keys.size and idx[name]["n_kmers"] == nk


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_matches_reference_fixture(path):
    text, W, k, keys, counts, nk = load(path)
    got_k, got_c, got_n = pyoracle.count(text, W, k)
    assert got_n == nk
    assert np.array_equal(got_k, keys)
    assert np.array_equal(got_c, counts)
    assert int(counts.astype(np.uint64).sum()) == nk


@pytest.mark.parametrize("path", FIXTURES[:6], ids=[os.path.basename(p)[:-4] for p in FIXTURES[:6]])
def test_port_matches_reference_fixture(path):
    text, W, k, keys, counts, nk = load(path)
    for pes in (1, 3):
        (gk, gc, gn), secs = pyoracle.dakc_port(text, W, k, pes)
        assert gn == nk and np.array_equal(gk, keys) and np.array_equal(gc, counts)


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_count_mt_matches_reference_fixture(path):
    """The range-parallel checker (used at config size) reproduces every
    reference table, for several thread counts."""
    text, W, k, keys, counts, nk = load(path)
    for threads in (1, 3, 8):
        gk, gc, gn = pyoracle.count_mt(text, W, k, threads)
        assert gn == nk and np.array_equal(gk, keys) and np.array_equal(gc, counts)


def test_count_mt_equals_count_random():
    text = synth.random_lines(12, 4000, 100, b"ACGTACGTACGTN")
    for k in (1, 5, 6, 7, 13, 31, 32):
        ref = pyoracle.count(text, 100, k)
        got = pyoracle.count_mt(text, 100, k, 5)
        assert got[2] == ref[2] and np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert pyoracle.count_mt(b"", 10, 4)[2] == 0


def test_plain_1m_digest():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        ent = json.load(f)["cases"]["plain_1m"]
    rs = synth.plain_1m()
    assert hashlib.sha256(rs.text.tobytes()).hexdigest() == ent["text_sha256"]
    for keys, counts, nk in (pyoracle.count(rs.text, 150, 31), pyoracle.count_mt(rs.text, 150, 31)):
        assert nk == ent["n_kmers"] and keys.size == ent["n_distinct"]
        assert hashlib.sha256(keys.tobytes() + counts.tobytes()).hexdigest() == ent["table_sha256"]


def _with_one_more_zero(keys, counts):
    """The table plus one occurrence of k-mer 0."""
    keys = [int(x) for x in keys]
    counts = [int(x) for x in counts]
    if keys and keys[0] == 0:
        counts[0] += 1
    else:
        keys.insert(0, 0)
        counts.insert(0, 1)
    return keys, counts


def test_hitter1_record():
    """The reference built with HITTER=1 (the header default,
    common.hpp:42-44) gives the HITTER=0 table on every golden input but one.
    In edge_w20_k1 every k-mer of the PE reaches it as a heavy (k-mer, count)
    pair, so its light vector is empty; phase 2 still starts its run-length
    pass at element 0 of that vector (kcounter.cpp:334, 368-377) and counts one
    occurrence of k-mer 0.  The engine follows the HITTER=0 table."""
    with open(os.path.join(GOLDEN, "hitter1.json")) as f:
        rec = json.load(f)["cases"]
    assert set(rec) == {os.path.basename(p)[:-4] for p in FIXTURES}
    differing = []
    for name, runs in rec.items():
        text, W, k, keys, counts, nk = load(os.path.join(GOLDEN, name + ".npz"))
        for p, ent in runs.items():
            if ent["equals_hitter0"]:
                assert ent["table_sha256"] == hashlib.sha256(keys.tobytes() + counts.tobytes()).hexdigest()
                assert ent["n_kmers"] == nk
            else:
                differing.append(name)
                assert (ent["keys"], ent["counts"]) == _with_one_more_zero(keys, counts)
                assert ent["n_kmers"] == nk + 1
    assert differing == ["edge_w20_k1"]


@pytest.mark.skipif(not os.path.isdir(pyoracle.REFERENCE_TREE), reason="reference tree absent")
@pytest.mark.parametrize("name", ["reads_w150_k31", "skew_w150_k31", "edge_w20_k1"])
def test_hitter1_live(name):
    text, W, k, keys, counts, nk = load(os.path.join(GOLDEN, name + ".npz"))
    with open(os.path.join(GOLDEN, "hitter1.json")) as f:
        runs = json.load(f)["cases"][name]
    for p, ent in runs.items():
        (hk, hc, hn), _ = pyoracle.ref_table(text, W, k, pes=int(p), hitter=1)
        assert hashlib.sha256(hk.tobytes() + hc.tobytes()).hexdigest() == ent["table_sha256"]
        assert hn == ent["n_kmers"]


def test_known_answers():
    # hand-derived from the convention: C=0 A=1 T=2 G=3, MSB-first
    assert pyoracle.count(b"CAT\n", 3, 3)[0].tolist() == [6]
    assert pyoracle.count(b"GGG\n", 3, 3)[0].tolist() == [63]
    assert pyoracle.count(b"ACG\n", 3, 3)[0].tolist() == [19]
    assert pyoracle.count(b"CANTG\n", 5, 3)[0].size == 0
    assert pyoracle.count(b"CATMAAA\n", 7, 3)[0].tolist() == [6]
    assert pyoracle.count(b"G" * 32 + b"\n", 32, 32)[0].tolist() == [2 ** 64 - 1]
    keys, counts, nk = pyoracle.count(b"AAAAA\nAAAAA\n", 5, 3)
    assert keys.tolist() == [0b010101] and counts.tolist() == [6] and nk == 6


def test_code_table():
    t = pyoracle.code_table()
    expect = np.full(256, 0xFF, np.uint8)
    for chars, v in ((b"Cc", 0), (b"Aa", 1), (b"Tt", 2), (b"Gg", 3), (b"Mm", 0xF0)):
        for c in chars:
            expect[c] = v
    assert np.array_equal(t, expect)


def test_framing():
    W = 5
    assert pyoracle.num_lines(b"", W) == 0
    assert pyoracle.num_lines(b"ACGTA\nACGTA\n", W) == 2
    assert pyoracle.num_lines(b"ACGTA\nACGTA", W) == 2       # last terminator missing
    assert pyoracle.num_lines(b"ACGTA\nACG", W) == -1        # partial line
    assert pyoracle.num_lines(b"ACGTA\n\0CGTA\nACGTA\n", W) == 1  # NUL-led line stops parsing
    assert pyoracle.num_lines(b"\0CGTA\nACGTA\n", W) == 2    # line 0 is always parsed
    with pytest.raises(pyoracle.OracleError):
        pyoracle.count(b"ACGTA\nACG", W, 3)


def test_k1_last_run_rule():
    # a final run starting at W-1 is not emitted (kcounter_funcs.cpp:97)
    assert pyoracle.count(b"ACGTNA\n", 6, 1)[2] == 4
    assert pyoracle.count(b"ACGTAA\n", 6, 1)[2] == 6
    assert pyoracle.count(b"A\n", 1, 1)[2] == 0


def test_port_equals_oracle_random():
    text = synth.random_lines(11, 3000, 150, b"ACGTACGTACGTN")
    ref = pyoracle.count(text, 150, 21)
    for pes in (1, 2, 5, 8):
        (k, c, n), _ = pyoracle.dakc_port(text, 150, 21, pes)
        assert n == ref[2] and np.array_equal(k, ref[0]) and np.array_equal(c, ref[1])


def test_murmur_owner_spreads_keys():
    # DAKC's owner hash (kcounter.cpp:29-54) must spread consecutive keys over PEs
    owners = [pyoracle.murmur64a(i) % 16 for i in range(4096)]
    counts = np.bincount(owners, minlength=16)
    assert counts.min() > 180 and counts.max() < 340


def _reference_available():
    return pyoracle.ref_binary(31, 150, 0, build=True) is not None


@pytest.mark.skipif(not os.path.isdir(pyoracle.REFERENCE_TREE), reason="reference tree absent")
def test_oracle_matches_live_reference():
    assert _reference_available()
    g = synth.genome_uniform(51, 100_000)
    text = synth.reads(52, g, 3000, 150, 150, 150, rc_frac=0.5, err_rate=0.02)
    ref, out = pyoracle.ref_table(text, 150, 31, pes=3)
    mine = pyoracle.count(text, 150, 31)
    assert "kmer counting time" in out
    assert ref[2] == mine[2] and np.array_equal(ref[0], mine[0]) and np.array_equal(ref[1], mine[1])


def test_pakman_histogram_cutoff_known_answer():
    # counts 1,1,1,2,3,3,5,7 with 6 buckets: hist = [0,3,1,2,0,1]; first min of
    # hist[1:] is bucket 4 (hist 0), so k-mers with count >= 4 are kept
    hist, mb = pyoracle.pakman_histogram_cutoff([1, 1, 1, 2, 3, 3, 5, 7], 6)
    assert list(hist) == [0, 3, 1, 2, 0, 1]
    assert mb == 4
    # ties: the first minimum wins (std::min_element)
    hist, mb = pyoracle.pakman_histogram_cutoff([1, 2, 3, 3], 4)
    assert list(hist) == [0, 1, 1, 2] and mb == 1
    assert pyoracle.pakman_histogram_cutoff([5, 6], 1)[1] == 0


def test_fq2txt_known_answer():
    fq = b"@r1\nACGT\n+\nIIII\n@r2\nAC GTA\n+\nIIIII\n@r3\nA\n+\nI"
    txt, w = pyoracle.fq2txt(fq)
    assert w == 6
    assert txt == b"ACGTMM\nACMGTA\nAMMMMM\n"


def test_pakman_kmers_known_answer():
    # A=0 C=1 T=2 G=3 via (byte >> 1) & 7; k = 3
    fa = b"junk\n>h1\nACGTA\n>h2\nGG\n>h3\nTTT"
    got = pyoracle.pakman_kmers(fa, 3)
    enc = lambda s: sum(((b >> 1) & 7) << (2 * (len(s) - 1 - i)) for i, b in enumerate(s))
    assert got.tolist() == [enc(b"ACG"), enc(b"CGT"), enc(b"GTA"), enc(b"TTT")]
    # 'N' (0x4E -> 7) is OR'ed into the window as PakMan* does, not skipped
    got = pyoracle.pakman_kmers(b">h\nANC\n", 2)
    assert got.tolist() == [((0 << 2) | 7) & 15, ((7 << 2) | 1) & 15]
    assert pyoracle.format_lines(fa, "fasta") == [b"ACGTA", b"GG", b"TTT"]
    assert pyoracle.format_lines(b"x\n>a\nC\n", "fasta") == [b"C"]


FORMAT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "formats", "formats_*.npz")))


@pytest.mark.parametrize("path", FORMAT_FIXTURES, ids=[os.path.basename(p)[:-4] for p in FORMAT_FIXTURES])
def test_format_restatements_match_reference_runs(path):
    """The restatements behind the read-format rows reproduce what the
    reference's own code produced on the same input: fq2txtmaker.sh's text
    (run with bash/awk/sed), DAKC's table of that text, and PakMan*'s table of
    fq2famaker.sh's FASTA (kmer_counting.cpp compiled unmodified, one rank)."""
    z = np.load(path)
    fq, txt, fa, W = z["fastq"].tobytes(), z["txt"].tobytes(), z["fa"].tobytes(), int(z["W"])
    with open(os.path.join(GOLDEN, "formats", "formats.json")) as f:
        ent = json.load(f)["cases"][os.path.basename(path)[:-4]]
    assert hashlib.sha256(fq).hexdigest() == ent["fastq_sha256"]
    got_txt, w = pyoracle.fq2txt(fq)
    assert w == W and got_txt == txt
    for k in (21, 31):
        keys, counts, nk = pyoracle.count(np.frombuffer(txt, np.uint8), W, k)
        assert nk == int(z[f"dakc_nk_k{k}"])
        assert np.array_equal(keys, z[f"dakc_keys_k{k}"]) and np.array_equal(counts, z[f"dakc_counts_k{k}"])
        pk, pc, _ = pyoracle.table_of(pyoracle.pakman_kmers(fa, k))
        assert np.array_equal(pk, z[f"pakman_keys_k{k}"]) and np.array_equal(pc, z[f"pakman_counts_k{k}"])

"""GPU engine vs the CPU oracle, bit for bit, through the C ABI.

Every case compares the full table (sorted distinct k-mers, their uint32
counts) and the occurrence total.  Integer work: the bar is exact equality.
"""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu

VARIANTS = [dk.VARIANT_SORT, dk.VARIANT_HASH]


def check(engine, text, W, k, variant=dk.VARIANT_SORT):
    got = engine.count(text, W, k, variant)
    keys, counts, nk = pyoracle.count(text, W, k)
    assert got.n_kmers == nk
    assert got.kmers.size == keys.size, (got.kmers.size, keys.size)
    assert np.array_equal(got.kmers, keys)
    assert np.array_equal(got.counts, counts)
    return got


def lines(*rows, W):
    out = b""
    for r in rows:
        assert len(r) <= W
        out += r + b"M" * (W - len(r)) + b"\n"
    return out


# ------------------------------------------- the reference's own tables
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_reference_fixture(engine, variant, path):
    z = np.load(path)
    got = engine.count(z["text"], int(z["W"]), int(z["k"]), variant)
    assert got.n_kmers == int(z["n_kmers"])
    assert np.array_equal(got.kmers, z["keys"])
    assert np.array_equal(got.counts, z["counts"])


@pytest.mark.parametrize("variant", VARIANTS)
def test_reference_digest_plain_1m(engine, variant):
    with open(os.path.join(GOLDEN, "index.json")) as f:
        ent = json.load(f)["cases"]["plain_1m"]
    rs = synth.plain_1m()
    got = engine.count(rs.text, 150, 31, variant)
    h = hashlib.sha256(got.kmers.tobytes() + got.counts.tobytes()).hexdigest()
    assert got.n_kmers == ent["n_kmers"] and h == ent["table_sha256"]


# ------------------------------------------------------------ known answers
@pytest.mark.parametrize("variant", VARIANTS)
def test_known_answers(engine, variant):
    assert engine.count(b"CAT\n", 3, 3, variant).kmers.tolist() == [6]
    assert engine.count(b"GGG\n", 3, 3, variant).kmers.tolist() == [63]
    assert engine.count(b"ACG\n", 3, 3, variant).kmers.tolist() == [19]
    assert engine.count(b"CANTG\n", 5, 3, variant).kmers.size == 0
    r = engine.count(b"CATMAAA\n", 7, 3, variant)
    assert r.kmers.tolist() == [6] and r.counts.tolist() == [1]
    r = engine.count(b"G" * 32 + b"\n", 32, 32, variant)
    assert r.kmers.tolist() == [0xFFFFFFFFFFFFFFFF]


@pytest.mark.parametrize("variant", VARIANTS)
def test_empty_and_short(engine, variant):
    for text, W, k in [(b"", 150, 31), (b"ACG\n", 3, 4), (b"NNNN\n", 4, 2), (b"MMMM\n", 4, 1),
                       (b"AC\nGT\n", 2, 3)]:
        r = engine.count(text, W, k, variant)
        assert r.kmers.size == 0 and r.n_kmers == 0


@pytest.mark.parametrize("variant", VARIANTS)
def test_framing_rules(engine, variant):
    W = 20
    rows = [b"ACGTACGTACGTACGTACGT", b"acgtNacgtacgtACGT", b"ACGTACGM", b"ACGTAC\nGTAC",
            b"AAAAAAAAAAAAAAAAAAAA", b"TTTT TTTT-TTTTTTT", b"CCCCMCCCCCCCCC"]
    text = lines(*rows, W=W)
    for k in (1, 2, 3, 5, 8, 13, 20):
        check(engine, text, W, k, variant)
    # last terminator missing
    check(engine, text[:-1], W, 5, variant)
    # the terminator byte is never examined
    t2 = bytearray(text)
    t2[W] = ord("A")
    check(engine, bytes(t2), W, 5, variant)


@pytest.mark.parametrize("variant", VARIANTS)
def test_k1_last_run_rule(engine, variant):
    # k=1: a final run starting at W-1 is dropped (kcounter_funcs.cpp:97)
    W = 6
    text = lines(b"ACGTNA", b"ACGTAA", b"NNNNNA", b"ACGTAN", b"ACMGTA", W=W)
    got = check(engine, text, W, 1, variant)
    assert got.n_kmers == 4 + 6 + 0 + 5 + 2
    check(engine, b"A\nC\nG\n", 1, 1, variant)  # W=1: nothing is emitted


@pytest.mark.parametrize("variant", VARIANTS)
def test_nul_line_stops_parsing(engine, variant):
    W = 10
    rows = [b"ACGTACGTAC", b"CCCCCCCCCC", b"\0GGGGGGGGG", b"TTTTTTTTTT"]
    text = lines(*rows, W=W)
    got = check(engine, text, W, 4, variant)
    assert got.n_kmers == 14  # lines 0 and 1 only
    # NUL inside a line is just a break; NUL as the first byte of line 0 too
    text = lines(b"\0CGTACGTAC", b"CCCC\0CCCCC", W=W)
    check(engine, text, W, 4, variant)


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("W,k", [(1, 1), (2, 1), (31, 31), (32, 31), (33, 17), (64, 32),
                                 (100, 21), (150, 31), (150, 17), (250, 31), (257, 25),
                                 (500, 31), (1000, 15)])
def test_random_shapes(engine, variant, W, k):
    text = synth.random_lines(W * 7 + k, 3000, W, b"ACGTACGTACGTacgtNM")
    check(engine, text, W, k, variant)


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("k", [1, 2, 5, 6, 7, 11, 12, 13, 16, 21, 27, 32])
def test_k_sweep(engine, variant, k):
    g = synth.genome_uniform(100 + k, 50_000)
    text = synth.reads(200 + k, g, 5000, 80, 100, 100, rc_frac=0.5, err_rate=0.01)
    check(engine, text, 100, k, variant)


@pytest.mark.parametrize("variant", VARIANTS)
def test_plain_1m_workload(engine, variant):
    rs = synth.plain_1m()
    got = check(engine, rs.text, rs.line_width, rs.k, variant)
    assert got.n_kmers == 12_000_000


@pytest.mark.parametrize("variant", VARIANTS)
def test_skew_heavy_hitters(engine, variant):
    # a few reads repeated very many times: giant buckets, dense and deep paths
    W = 150
    g = synth.genome_uniform(7, 20_000)
    hot = synth.reads(8, g, 3, 150, 150, W, rc_frac=0.0)
    bg = synth.reads(9, g, 20_000, 150, 150, W, rc_frac=0.5, err_rate=0.01)
    text = np.concatenate([np.tile(hot, 40_000), bg])
    got = check(engine, text, W, 31, variant)
    assert got.counts.max() >= 40_000
    # one k-mer only: every count lands in one key
    text = np.frombuffer(lines(b"A" * 150, W=150) * 20_000, dtype=np.uint8)
    got = check(engine, text, W, 31, variant)
    assert got.kmers.size == 1 and got.counts[0] == 120 * 20_000


@pytest.mark.parametrize("variant", VARIANTS)
def test_one_kmer_dominates_a_normal_bin(engine, variant):
    """A k-mer with about 2,000 copies among 24 M background k-mers: its bin is
    a normal one (its node is far from half of its parent), so the packed
    table takes it, and its copies add to one entry lane by lane."""
    W = 150
    g = synth.genome_uniform(31, 3_000_000)
    bg = synth.reads(32, g, 200_000, 150, 150, W, rc_frac=0.5, err_rate=0.01)
    hot = np.frombuffer(lines(b"A" * 150, W=150) * 17, dtype=np.uint8)
    text = np.concatenate([bg[: 1000 * (W + 1)], hot, bg[1000 * (W + 1):]])
    got = check(engine, text, W, 31, variant)
    a31 = int("01" * 31, 2)
    i = int(np.searchsorted(got.kmers, np.uint64(a31)))
    assert got.kmers[i] == a31 and got.counts[i] >= 17 * 120


@pytest.mark.parametrize("variant", VARIANTS)
def test_two_partition_levels(engine, variant):
    # > 4096 * 6144 k-mers forces the 8-bit partition level below level 1
    g = synth.genome_uniform(21, 30_000_000)
    text = synth.reads(22, g, 300_000, 150, 150, 150, rc_frac=0.5, err_rate=0.005)
    check(engine, text, 150, 31, variant)
    st = engine.stats()
    assert st["partition_levels"] >= 2


def test_table_device_residency(engine):
    text = synth.random_lines(5, 1000, 150)
    d = dk.Engine.desc(150, 21, dk.VARIANT_SORT, dk.RESIDENT_DEVICE)
    ptr = text.ctypes.data
    t = engine.count_raw(ptr, text.size, d)
    try:
        assert t.on_device == 1 and t.n > 0
    finally:
        engine.free_table(t)


def test_invalid_arguments(engine):
    for W, k, n in [(150, 0, 151), (150, 33, 151), (0, 3, 1), (150, 31, 100)]:
        with pytest.raises(dk.DkError) as e:
            engine.count(b"A" * n, W, k)
        assert e.value.status == dk.DK_ERR_INVALID_ARG


@pytest.mark.parametrize("variant", VARIANTS)
def test_hot_kmer_needs_many_partition_levels(engine, variant):
    """One 31-mer 20,000 times (just above a bin's capacity) among random
    reads: its node splits by only a couple of bits per level, so the
    partition runs many levels (more than 16) before it is counted densely."""
    rng = np.random.Generator(np.random.PCG64(77))
    hot = rng.choice(np.frombuffer(b"ACGT", np.uint8), 31)
    W = 31
    lines = np.empty((20_000 + 30_000, W + 1), np.uint8)
    lines[:20_000, :W] = hot
    lines[20_000:, :W] = rng.choice(np.frombuffer(b"ACGT", np.uint8), (30_000, W))
    lines[:, W] = ord("\n")
    rng.shuffle(lines[:-1])
    text = lines.reshape(-1)
    keys, counts, nk = pyoracle.count(text, W, 31)
    r = engine.count(text, W, 31, variant)
    st = engine.stats()
    assert r.n_kmers == nk and np.array_equal(r.kmers, keys) and np.array_equal(r.counts, counts)
    assert int(counts.max()) >= 20_000
    if variant == dk.VARIANT_HASH:
        # the hot node is counted whole by one hash bin, a level or two down
        assert st["n_bins_big"] >= 1 and st["n_bins_retried"] == 0
        assert st["partition_levels"] <= 4
    else:
        assert st["partition_levels"] > 16


@pytest.mark.parametrize("variant", VARIANTS)
def test_skewed_node_with_many_distinct_kmers_is_repartitioned(engine, variant):
    """60,000 distinct 31-mers behind one 20-base prefix, a hot 31-mer with the
    same prefix and random reads: the prefix's node keeps most of its
    parent's keys at every level, so the hash variant tries it as one big bin,
    finds too many distinct keys and partitions it further, round after round
    until the prefix is spent."""
    rng = np.random.Generator(np.random.PCG64(78))
    acgt = np.frombuffer(b"ACGT", np.uint8)
    W = 31
    prefix = rng.choice(acgt, 20)
    lines = np.empty((60_000 + 5_000 + 30_000, W + 1), np.uint8)
    lines[:65_000, :20] = prefix
    lines[:60_000, 20:W] = rng.choice(acgt, (60_000, W - 20))
    lines[60_000:65_000, 20:W] = rng.choice(acgt, W - 20)
    lines[65_000:, :W] = rng.choice(acgt, (30_000, W))
    lines[:, W] = ord("\n")
    rng.shuffle(lines)
    text = lines.reshape(-1)
    keys, counts, nk = pyoracle.count(text, W, 31)
    r = engine.count(text, W, 31, variant)
    st = engine.stats()
    assert r.n_kmers == nk and np.array_equal(r.kmers, keys) and np.array_equal(r.counts, counts)
    if variant == dk.VARIANT_HASH:
        assert st["n_bins_retried"] >= 2


@pytest.fixture(scope="module")
def streaming_engine():
    with dk.Engine(0, flags=dk.FLAG_STREAM_ALL) as e:
        yield e


@pytest.mark.parametrize("variant", VARIANTS)
def test_streamed_host_table(streaming_engine, variant):
    """A host table copied out group by group while the count runs is the
    oracle's table."""
    rs = synth.plain_1m()
    text = rs.text[: 40_000 * (rs.line_width + 1)]
    check(streaming_engine, text, rs.line_width, rs.k, variant)
    st = streaming_engine.stats()
    assert st["n_groups"] >= 2 and st["table_streamed"] == 1


@pytest.mark.parametrize("variant", VARIANTS)
def test_streamed_table_size_estimate_too_small(variant):
    """The first group holds ten k-mers copied 10,000 times each, the rest are
    random: the host table sized from the first group is too small, so the
    table is copied after the count instead, and is still exact."""
    rng = np.random.Generator(np.random.PCG64(79))
    acgt = np.frombuffer(b"ACGT", np.uint8)
    W = 31
    hot = rng.choice(acgt, (10, W))
    hot[:, :4] = ord("C")  # C = 0: the smallest keys, first group
    lines = np.empty((100_000 + 100_000, W + 1), np.uint8)
    lines[:100_000, :W] = hot[np.arange(100_000) % 10]
    lines[100_000:, :W] = rng.choice(acgt, (100_000, W))
    lines[:, W] = ord("\n")
    rng.shuffle(lines)
    # a fresh context: no pooled host table larger than the estimate
    with dk.Engine(0, flags=dk.FLAG_STREAM_ALL) as e:
        check(e, lines.reshape(-1), W, 31, variant)
        st = e.stats()
    assert st["n_groups"] >= 2 and st["table_streamed"] == 0


def _reads_68mb(seed):
    g = synth.genome_uniform(seed, 2_000_000)
    return synth.reads(seed + 1, g, 450_000, 150, 150, 150, rc_frac=0.5, err_rate=0.01)


@pytest.mark.parametrize("nul_line", [None, 200_001])
def test_chunked_upload_equals_single_upload(engine, nul_line):
    """Page-locked reads of 64 MB or more upload in chunks of lines, each
    counted as soon as it lands; so do pageable reads where the device reads
    them in place.  Both tables equal the one counted from the same bytes
    staged through page-locked slots and uploaded whole, also when a NUL-led
    line in the middle of a chunk ends the read set there."""
    text = _reads_68mb(81)
    if nul_line is not None:
        text[nul_line * 151] = 0
    pin = dk.PinnedBuffer(text.size)
    try:
        pin.array[:] = text
        a = engine.count(pin.array, 150, 31, dk.VARIANT_HASH)
        chunks = engine.stats()["upload_chunks"]
        p = engine.count(text, 150, 31, dk.VARIANT_HASH)
        st_p = engine.stats()
    finally:
        pin.free()
    with dk.Engine(0, flags=dk.FLAG_STAGE_PAGEABLE) as staged:
        b = staged.count(text, 150, 31, dk.VARIANT_HASH)
        st_b = staged.stats()
    assert st_b["upload_chunks"] == 0 and st_b["upload_in_place"] == 0
    assert st_p["upload_chunks"] == (chunks if st_p["upload_in_place"] else 0)
    assert chunks >= 2
    for r in (a, p):
        assert r.n_kmers == b.n_kmers and np.array_equal(r.kmers, b.kmers)
        assert np.array_equal(r.counts, b.counts)
    assert int(a.counts.sum(dtype=np.uint64)) == a.n_kmers
    if nul_line is not None:
        assert a.n_kmers == nul_line * 120


def _count_conv(engine, text, W, k, conv, variant):
    d = dk.Engine.desc(W, k, variant)
    d.convention = conv
    ptr, n, keep = dk._buf_ptr(text)
    t = engine.count_raw(ptr, n, d)
    try:
        nd = int(t.n)
        return (np.ctypeslib.as_array(t.kmers, shape=(nd,)).copy(),
                np.ctypeslib.as_array(t.counts, shape=(nd,)).copy(), int(t.n_kmers))
    finally:
        engine.free_table(t)


@pytest.mark.parametrize("conv,variant", [(dk.CONV_PAKMAN, dk.VARIANT_HASH),
                                          (dk.CONV_DAKC, dk.VARIANT_SORT)])
def test_chunked_upload_other_convention_and_variant(engine, conv, variant):
    """The chunked upload under PakMan*'s convention and under the sort
    variant equals the single upload of the same bytes."""
    text = _reads_68mb(82)
    pin = dk.PinnedBuffer(text.size)
    try:
        pin.array[:] = text
        a = _count_conv(engine, pin.array, 150, 31, conv, variant)
        assert engine.stats()["upload_chunks"] >= 2
    finally:
        pin.free()
    with dk.Engine(0, flags=dk.FLAG_STAGE_PAGEABLE) as staged:
        b = _count_conv(staged, text, 150, 31, conv, variant)
        assert staged.stats()["upload_chunks"] == 0
    assert a[2] == b[2] and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert int(a[1].sum(dtype=np.uint64)) == a[2]


@pytest.mark.parametrize("variant", VARIANTS)
def test_streamed_and_chunked_together(variant):
    """A page-locked read set uploaded in chunks whose table also streams out
    in groups equals the single-upload, single-copy count of the same bytes."""
    text = _reads_68mb(83)
    with dk.Engine(0, flags=dk.FLAG_STREAM_ALL) as e1, \
            dk.Engine(0, flags=dk.FLAG_STAGE_PAGEABLE) as e2:
        pin = dk.PinnedBuffer(text.size)
        try:
            pin.array[:] = text
            a = e1.count(pin.array, 150, 31, variant)
            st = e1.stats()
        finally:
            pin.free()
        b = e2.count(text, 150, 31, variant)
        st2 = e2.stats()
    assert st["upload_chunks"] >= 2 and st["table_streamed"] == 1 and st["n_groups"] >= 2
    assert st2["upload_chunks"] == 0 and st2["table_streamed"] == 0
    assert a.n_kmers == b.n_kmers and np.array_equal(a.kmers, b.kmers)
    assert np.array_equal(a.counts, b.counts)


def test_failed_chunked_count_leaves_the_context_usable():
    """A count that does not fit the context's memory budget fails with an
    admission or memory status after its chunked upload has started; the
    same context then counts other reads exactly."""
    text = _reads_68mb(84)
    with dk.Engine(0, mem_budget=256 << 20) as e:
        pin = dk.PinnedBuffer(text.size)
        try:
            pin.array[:] = text
            with pytest.raises(dk.DkError) as ei:
                e.count(pin.array, 150, 31, dk.VARIANT_HASH)
            assert ei.value.status in (dk.DK_ERR_ADMISSION, dk.DK_ERR_OOM)
            small = pin.array[: 20_000 * 151].copy()  # outlives the page-locked buffer
        finally:
            pin.free()
        check(e, small, 150, 31, dk.VARIANT_HASH)


def test_chunked_upload_with_lines_shorter_than_k(engine):
    """A 64 MB page-locked read set whose lines are shorter than k has no
    k-mers; the call returns an empty table after its chunked upload ends,
    and the context counts the next reads exactly."""
    W = 20
    n_lines = (70 << 20) // (W + 1)
    text = np.full((n_lines, W + 1), ord("A"), np.uint8)
    text[:, W] = ord("\n")
    pin = dk.PinnedBuffer(text.size)
    try:
        pin.array[:] = text.reshape(-1)
        r = engine.count(pin.array, W, 31)
        assert r.n_kmers == 0 and r.kmers.size == 0
    finally:
        pin.free()
    small = _reads_68mb(85)[: 5_000 * 151]
    check(engine, small, 150, 31)


@pytest.mark.parametrize("variant", VARIANTS)
def test_repeats_in_bins_with_many_free_bits(engine, variant):
    """A small read set is split by few bits, so its bins keep most of the
    key's bits free and the packed table's count field is narrow: a k-mer
    repeated past that field's limit sends its bin to the general bin kernel,
    and the table stays exact."""
    rng = np.random.Generator(np.random.PCG64(83))
    acgt = np.frombuffer(b"ACGT", np.uint8)
    W = 40
    lines = np.empty((3000, W + 1), np.uint8)
    lines[:, :W] = rng.choice(acgt, (3000, W))
    lines[:1000, :W] = lines[0, :W]          # one read, 1,000 times: its 10 k-mers repeat
    lines[:, W] = ord("\n")
    rng.shuffle(lines)
    text = lines.reshape(-1)
    got = check(engine, text, W, 31, variant)
    assert int(got.counts.max()) >= 1000
    if variant == dk.VARIANT_HASH:
        st = engine.stats()
        assert st["n_bins_packed"] + st["n_bins_fallback"] >= 1

"""Pageable reads read in place by the device.

On a host whose memory the GPU reads through the host's own page tables
(Grace: coherent chip-to-chip access), dk_count copies pageable reads into
device memory with a kernel instead of staging them through page-locked slots
with host threads.  The reference's caller hands the counter a malloc'd
buffer (dakc/src/fqreader/fqreader.cpp:59, dakc/src/main/main.cpp:42-49), so
this is the drop-in path.  The copy takes any alignment of either side: these
tests put the reads at every offset inside a 16-byte word, in small reads
(one copy), in chunked reads (each chunk counted as it lands) and in batched
read sets packed back to back, and compare with the oracle and with the
staged path.
"""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _at_offset(text: np.ndarray, off: int) -> np.ndarray:
    """The same bytes, starting `off` bytes past a 64-byte boundary."""
    buf = np.empty(text.size + 128, np.uint8)
    base = (-buf.ctypes.data) % 64
    view = buf[base + off: base + off + text.size]
    view[:] = text
    return view


def _count_view(eng, view, W, k, variant=dk.VARIANT_HASH):
    t = eng.count_raw(view.ctypes.data, view.size, dk.Engine.desc(W, k, variant))
    try:
        n = int(t.n)
        keys = np.ctypeslib.as_array(t.kmers, shape=(n,)).copy() if n else np.zeros(0, np.uint64)
        cnts = np.ctypeslib.as_array(t.counts, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        return keys, cnts, int(t.n_kmers)
    finally:
        eng.free_table(t)


@pytest.fixture(scope="module")
def engine():
    with dk.Engine(0) as eng:
        yield eng


def test_every_source_offset_small_reads(engine):
    """One copy of a small read set, from each of the 16 offsets in a word;
    sizes that end inside a word."""
    g = synth.genome_uniform(301, 300_000)
    text = synth.reads(302, g, 3_001, 150, 150, 150, rc_frac=0.5, err_rate=0.01)
    ref = pyoracle.count(text, 150, 31)
    for off in range(16):
        got = _count_view(engine, _at_offset(text, off), 150, 31)
        st = engine.stats()
        assert got[2] == ref[2] and np.array_equal(got[0], ref[0]), off
        assert np.array_equal(got[1], ref[1]), off
    assert st["upload_in_place"] in (0, 1)


def test_one_short_line_at_odd_offsets(engine):
    """Reads of fewer bytes than one 16-byte word, and of one word and a few
    bytes, at odd offsets: the copy writes only the bytes of the range."""
    for W, k in ((9, 5), (20, 7)):
        line = np.frombuffer(b"ACGTTGCAAGCTTAGGCATC"[:W] + b"\n", np.uint8).copy()
        ref = pyoracle.count(line, W, k)
        for off in (1, 7, 15):
            got = _count_view(engine, _at_offset(line, off), W, k)
            assert got[2] == ref[2] and np.array_equal(got[0], ref[0])
            assert np.array_equal(got[1], ref[1])


@pytest.mark.parametrize("off", [0, 5, 12])
def test_chunked_pageable_reads_at_offsets(engine, off):
    """A 68 MB pageable read set is read in place chunk by chunk (each chunk
    counted as it lands) from an aligned and from misaligned starts; the
    table equals the oracle's."""
    g = synth.genome_uniform(311, 2_000_000)
    text = synth.reads(312, g, 450_000, 150, 150, 150, rc_frac=0.5, err_rate=0.01)
    view = _at_offset(text, off)
    got = _count_view(engine, view, 150, 31)
    st = engine.stats()
    if st["upload_in_place"]:
        assert st["upload_chunks"] >= 2
    ref = pyoracle.count(text, 150, 31)
    assert got[2] == ref[2] and np.array_equal(got[0], ref[0])
    assert np.array_equal(got[1], ref[1])


@pytest.mark.parametrize("flags", [0, dk.FLAG_STAGE_PAGEABLE])
def test_batch_jobs_packed_back_to_back(flags):
    """Read sets that sit back to back in one pageable buffer, each starting
    at an arbitrary byte (and landing at an arbitrary byte of the wave's
    device buffer): every job's table equals the oracle's."""
    texts = [synth.random_lines(400 + j, 1 + (j * 37) % 90, 250) for j in range(40)]
    blob = np.concatenate([np.zeros(3, np.uint8)] + texts)
    views, pos = [], 3
    for t in texts:
        views.append(blob[pos: pos + t.size])
        pos += t.size
    with dk.Engine(0, mem_budget=64 << 20, flags=flags) as eng:
        got = eng.count_batch(views, 250, 31, dk.VARIANT_HASH)
    for j, t in enumerate(texts):
        keys, counts, nk = pyoracle.count(t, 250, 31)
        assert got[j].n_kmers == nk and np.array_equal(got[j].kmers, keys), j
        assert np.array_equal(got[j].counts, counts), j


def test_unmapped_reads_are_refused(engine):
    """Reads at host addresses this process no longer maps (a freed buffer)
    are refused with DK_ERR_INVALID_ARG before any kernel reads them, and the
    context counts the next reads exactly.  Only where the device reads
    pageable memory in place: the staged path copies on the host."""
    import ctypes
    import mmap
    text = synth.random_lines(501, 2_000, 150)
    engine.count(text, 150, 31)
    if not engine.stats()["upload_in_place"]:
        pytest.skip("pageable reads are staged on this host")
    libc = ctypes.CDLL(None, use_errno=True)
    libc.mmap.restype = ctypes.c_void_p
    libc.mmap.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                          ctypes.c_int, ctypes.c_long]
    libc.munmap.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    size = 80 << 20  # above the size read in chunks
    addr = libc.mmap(None, size, mmap.PROT_READ | mmap.PROT_WRITE,
                     mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS, -1, 0)
    assert addr not in (None, ctypes.c_void_p(-1).value)
    assert libc.munmap(addr, size) == 0
    nbytes = (size // 151) * 151
    for n in (151 * 10, nbytes):
        with pytest.raises(dk.DkError) as e:
            engine.count_raw(addr, n, dk.Engine.desc(150, 31))
        assert e.value.status == dk.DK_ERR_INVALID_ARG
    check_text = synth.random_lines(502, 3_000, 150)
    got = engine.count(check_text, 150, 31)
    keys, counts, nk = pyoracle.count(check_text, 150, 31)
    assert got.n_kmers == nk and np.array_equal(got.kmers, keys)
    assert np.array_equal(got.counts, counts)


def test_mapped_but_not_resident_reads_are_staged(engine):
    """Pageable reads whose pages are mapped but not all resident (here: an
    anonymous mapping whose second half was never touched) are staged through
    host threads, not read in place; the untouched half reads as zeros, so
    the read set ends at its first NUL-led line, as in the reference."""
    import ctypes
    import mmap
    W, n_lines = 150, 4000
    text = synth.random_lines(601, n_lines, W)
    half = (n_lines // 2) * (W + 1)
    buf = mmap.mmap(-1, text.size)            # untouched pages are not resident
    buf[:half] = text[:half].tobytes()
    view = ctypes.c_char.from_buffer(buf)     # keeps the mapping exported while in use
    t = engine.count_raw(ctypes.addressof(view), text.size, dk.Engine.desc(W, 31))
    try:
        n = int(t.n)
        keys = np.ctypeslib.as_array(t.kmers, shape=(n,)).copy()
        counts = np.ctypeslib.as_array(t.counts, shape=(n,)).copy()
        nk = int(t.n_kmers)
    finally:
        engine.free_table(t)
    assert engine.stats()["upload_in_place"] == 0
    ref = pyoracle.count(text[:half], W, 31)
    assert nk == ref[2] and np.array_equal(keys, ref[0]) and np.array_equal(counts, ref[1])
    del view
    buf.close()

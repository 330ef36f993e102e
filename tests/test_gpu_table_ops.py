"""Operations on finished tables (histogram / PakMan* cut-off, filter, lookup,
packed records) for host- and device-resident tables: exact against numpy and
the oracle's restatement of PakMan*'s cut-off."""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def reads():
    return synth.large_100m(genome_len=300_000).text   # 60,000 reads, 30x, repeats, errors


@pytest.mark.parametrize("residency", [dk.RESIDENT_HOST, dk.RESIDENT_DEVICE])
def test_histogram_filter_lookup_pairs(engine, reads, residency):
    keys, counts, nk = pyoracle.count(reads, 150, 31)
    t = engine.count_table(reads, 150, 31, dk.VARIANT_HASH, residency)
    try:
        assert int(t.n) == keys.size and int(t.on_device) == (residency == dk.RESIDENT_DEVICE)
        for nb in (1, 2, 40, 100, 256, 257, 20000):  # per-lane columns up to 256 buckets
            hist, mb = engine.histogram(t, nb)
            ref_hist, ref_mb = pyoracle.pakman_histogram_cutoff(counts, nb)
            assert np.array_equal(hist, ref_hist), nb
            assert mb == ref_mb, nb
        for min_count in (0, 1, 2, 5, 31, 1 << 30):
            f = engine.filter_table(t, min_count)
            try:
                keep = counts >= min_count
                assert int(f.n) == int(keep.sum())
                assert int(f.n_kmers) == int(counts[keep].sum(dtype=np.uint64))
                assert int(f.on_device) == int(t.on_device)
                if residency == dk.RESIDENT_HOST and int(f.n):
                    fk = np.ctypeslib.as_array(f.kmers, shape=(int(f.n),))
                    fc = np.ctypeslib.as_array(f.counts, shape=(int(f.n),))
                    assert np.array_equal(fk, keys[keep]) and np.array_equal(fc, counts[keep])
                if int(f.n):   # check the filtered table through a lookup too
                    q = keys[keep][:: max(1, int(f.n) // 500)]
                    assert np.array_equal(engine.lookup(f, q), counts[keep][:: max(1, int(f.n) // 500)])
            finally:
                engine.free_table(f)
        rng = np.random.Generator(np.random.PCG64(5))
        present = keys[rng.integers(0, keys.size, 5000)]
        absent = rng.integers(0, 1 << 62, 5000, dtype=np.uint64)
        q = np.concatenate([present, absent, keys[:1], keys[-1:], np.array([0, (1 << 62) - 1], np.uint64)])
        idx = np.searchsorted(keys, q)
        hit = (idx < keys.size) & (keys[np.minimum(idx, keys.size - 1)] == q)
        want = np.where(hit, counts[np.minimum(idx, keys.size - 1)], 0).astype(np.uint32)
        assert np.array_equal(engine.lookup(t, q), want)
        recs = engine.pairs(t)
        assert recs.dtype.itemsize == 12
        assert np.array_equal(recs["kmer"], keys) and np.array_equal(recs["count"], counts)
    finally:
        engine.free_table(t)


def test_operations_on_an_empty_table(engine):
    t = engine.count_table(b"", 150, 31)
    try:
        hist, mb = engine.histogram(t, 8)
        assert not hist.any() and mb == 1
        f = engine.filter_table(t, 2)
        assert int(f.n) == 0
        engine.free_table(f)
        assert engine.lookup(t, np.arange(5, dtype=np.uint64)).tolist() == [0] * 5
        assert engine.pairs(t).size == 0
    finally:
        engine.free_table(t)

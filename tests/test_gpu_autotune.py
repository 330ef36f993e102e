"""Autotuner (dk_autotune): it picks parameters inside their ranges, caches them
per input shape, and every tuned count stays exact (integer work)."""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def test_autotune_choice_and_exact_counts():
    rs = synth.large_100m(genome_len=1_000_000)          # 200,000 reads, 24 M k-mers
    small = rs.text[: 20_000 * 151]
    with dk.Engine(0) as eng:
        t = eng.autotune(rs.text, 150, 31)
        assert 1 <= t["l1_bits"] <= 12
        assert 0 < t["bin_target"] <= 6000
        assert t["variant"] in (dk.VARIANT_HASH, dk.VARIANT_SORT)
        assert t["candidates"] >= 4
        assert 0 < t["ms_device"] <= t["ms_auto"] * 1.0001
        tuned = eng.count(rs.text, 150, 31, dk.VARIANT_AUTO)   # takes the cached choice
        plain = eng.count(rs.text, 150, 31, dk.VARIANT_SORT)
        assert np.array_equal(tuned.kmers, plain.kmers)
        assert np.array_equal(tuned.counts, plain.counts)
        assert tuned.n_kmers == plain.n_kmers == int(plain.counts.sum(dtype=np.uint64))
        # a different shape is unaffected and still exact against the oracle
        keys, counts, nk = pyoracle.count(small, 150, 31)
        r = eng.count(small, 150, 31, dk.VARIANT_AUTO)
        assert np.array_equal(r.kmers, keys) and np.array_equal(r.counts, counts)
        eng.autotune_reset()
        again = eng.count(rs.text, 150, 31, dk.VARIANT_AUTO)
        assert np.array_equal(again.kmers, plain.kmers)

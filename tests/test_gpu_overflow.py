"""A k-mer that occurs 2^32 times or more.

The table's counts are uint32 (DAKC's count_t is u64, common.hpp:64-65): a
count that does not fit must end the call with DK_ERR_COUNT_OVERFLOW, never a
wrapped value.  One 31-mer repeated just below and just above 2^32 times
(lines of 150 'A's, 120 k-mers each; about 5.4 GB of reads and 86 GB of key
buffers on the device), under both bin variants; the context then counts the
next read set exactly.
"""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu

W, K = 150, 31
A31 = int("01" * 31, 2)  # 'A' = 1 in every 2-bit slot


def _device_lines_of_a(lines: int):
    import torch
    t = torch.full((lines, W + 1), ord("A"), dtype=torch.uint8, device="cuda")
    t[:, W] = ord("\n")
    flat = t.reshape(-1)
    pad = torch.zeros(flat.numel() + 64, dtype=torch.uint8, device="cuda")
    pad[: flat.numel()].copy_(flat)
    del t, flat
    torch.cuda.synchronize()
    return pad, lines * (W + 1)


@pytest.mark.parametrize("variant", [dk.VARIANT_HASH, dk.VARIANT_SORT])
def test_one_kmer_around_2_32_times(variant):
    import torch
    below = (1 << 32) // (W - K + 1) - 4_000    # 4,294,487,040 occurrences
    above = below + 10_000                      # 4,295,687,040 > 2^32
    torch.cuda.empty_cache()
    with dk.Engine(0) as eng:
        d_text, nbytes = _device_lines_of_a(below)
        t = eng.count_raw(d_text.data_ptr(), nbytes,
                          dk.Engine.desc(W, K, variant, dk.RESIDENT_HOST), on_device=True)
        try:
            assert int(t.n) == 1 and int(t.n_kmers) == below * (W - K + 1)
            assert int(t.kmers[0]) == A31 and int(t.counts[0]) == below * (W - K + 1)
        finally:
            eng.free_table(t)
        del d_text
        torch.cuda.empty_cache()

        d_text, nbytes = _device_lines_of_a(above)
        with pytest.raises(dk.DkError) as e:
            eng.count_raw(d_text.data_ptr(), nbytes,
                          dk.Engine.desc(W, K, variant, dk.RESIDENT_HOST), on_device=True)
        assert e.value.status == dk.DK_ERR_COUNT_OVERFLOW
        del d_text
        torch.cuda.empty_cache()

        # the context is still usable, and exact
        g = synth.genome_uniform(91, 200_000)
        text = synth.reads(92, g, 20_000, 150, 150, 150, rc_frac=0.5, err_rate=0.01)
        got = eng.count(text, W, K, variant)
        keys, counts, nk = pyoracle.count(text, W, K)
        assert got.n_kmers == nk and np.array_equal(got.kmers, keys)
        assert np.array_equal(got.counts, counts)

"""Batch waves whose tail runs as one CUDA graph.

dk_count_batch runs each wave's partition levels, bin count, tree offsets and
compact as one launch of a graph: the level loop is a conditional WHILE node
whose body plans the next level on the device, and the two tree passes are
WHILE nodes over the recorded levels.  These tests check that the graph's
tables equal the host-driven tail's and the oracle's:
- with several partition levels (large jobs split by one level-1 bit);
- under both bin variants;
- when a level outgrows the graph's buffers and the wave is counted again
  with the host-driven tail (the fallback, forced with minimal buffers);
- over several waves that reuse one graph (built once, replayed).
The reference counts each read set with its own counter
(dakc/src/kcounter/kcounter.hpp:84-99); these tables must equal those.
"""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _jobs(n, seed, max_reads):
    specs = synth.batch_specs(n, seed=seed, median=max_reads // 4, sigma=1.2, cap=max_reads)
    return [synth.batch_job_text(s, line_width=250, err_rate=0.005) for s in specs]


def _check_oracle(got, texts, W=250, k=31):
    for j, t in enumerate(texts):
        keys, counts, nk = pyoracle.count(t, W, k)
        assert got[j].n_kmers == nk, j
        assert np.array_equal(got[j].kmers, keys), j
        assert np.array_equal(got[j].counts, counts), j


@pytest.mark.parametrize("variant", [dk.VARIANT_HASH, dk.VARIANT_SORT])
def test_graph_equals_host_driven_tail(variant):
    texts = _jobs(48, seed=21, max_reads=6000)
    with dk.Engine(0, mem_budget=256 << 20) as g_eng, \
            dk.Engine(0, mem_budget=256 << 20, flags=dk.FLAG_NO_GRAPH) as h_eng:
        a = g_eng.count_batch(texts, 250, 31, variant)
        sa = g_eng.stats()
        b = h_eng.count_batch(texts, 250, 31, variant)
        sb = h_eng.stats()
    assert sa["n_waves"] >= 2 and sa["graph_waves"] + sa["graph_retries"] == sa["n_waves"]
    assert sa["graph_waves"] >= 1 and 1 <= sa["graph_builds"] <= sa["n_waves"]
    assert sb["graph_waves"] == 0 and sb["graph_builds"] == 0
    assert sa["n_kmers"] == sb["n_kmers"] and sa["n_distinct"] == sb["n_distinct"]
    for x, y in zip(a, b):
        assert x.n_kmers == y.n_kmers
        assert np.array_equal(x.kmers, y.kmers) and np.array_equal(x.counts, y.counts)
    _check_oracle(a, texts)


@pytest.mark.parametrize("variant", [dk.VARIANT_HASH, dk.VARIANT_SORT])
def test_graph_runs_several_levels(variant):
    """One level-1 bit per job leaves a 260,000-read job with level-1 nodes of
    ~1.6*10^7 keys: split 10 bits at a time, their children (~15,000 keys)
    split again, so the graph's level loop runs three levels (two that split,
    one that does not)."""
    g = synth.genome_uniform(611, 3_000_000)
    big = synth.reads(612, g, 260_000, 150, 150, 250, rc_frac=0.5, err_rate=0.01)
    small = _jobs(6, seed=22, max_reads=2000)
    texts = [big] + small
    with dk.Engine(0) as eng:
        got = eng.count_batch(texts, 250, 31, variant, l1_bits=1)
        st = eng.stats()
    assert st["graph_waves"] == st["n_waves"] and st["graph_retries"] == 0
    assert st["partition_levels"] >= 3
    _check_oracle(got, texts)


def test_graph_fallback_when_buffers_are_too_small():
    """With minimal graph buffers the levels of a large wave outgrow them: the
    wave is counted again with the host-driven tail, and its tables are the
    same."""
    g = synth.genome_uniform(621, 2_000_000)
    big = synth.reads(622, g, 120_000, 150, 150, 250, rc_frac=0.5, err_rate=0.01)
    texts = [big] + _jobs(10, seed=23, max_reads=3000)
    with dk.Engine(0, flags=dk.FLAG_GRAPH_MIN_BUFFERS) as eng:
        got = eng.count_batch(texts, 250, 31, dk.VARIANT_HASH, l1_bits=1)
        st = eng.stats()
    assert st["graph_retries"] >= 1
    _check_oracle(got, texts)

"""dk_count_batch: many read sets in one pipeline, each table bit-exact."""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def job_texts(n, seed=0, W=250, max_reads=3000):
    specs = synth.batch_specs(n, seed=seed + 4, median=400, sigma=1.5, cap=max_reads)
    assert sum(s.n_reads for s in specs) > 0
    return [synth.batch_job_text(s, line_width=W, err_rate=0.005) for s in specs]


@pytest.mark.parametrize("variant", [dk.VARIANT_SORT, dk.VARIANT_HASH])
def test_batch_matches_oracle_and_plain(engine, variant):
    texts = job_texts(40)
    texts[3] = np.zeros(0, np.uint8)                      # empty job
    texts[7] = texts[7][:-1]                              # last terminator missing
    texts[9] = synth.random_lines(3, 20, 250, b"N")       # no k-mers at all
    got = engine.count_batch(texts, 250, 31, variant)
    assert len(got) == len(texts)
    for j, t in enumerate(texts):
        keys, counts, nk = pyoracle.count(t, 250, 31)
        assert got[j].n_kmers == nk, j
        assert np.array_equal(got[j].kmers, keys), j
        assert np.array_equal(got[j].counts, counts), j
    # and equal to counting each job alone
    for j in (0, 5, 7, 20):
        alone = engine.count(texts[j], 250, 31, variant)
        assert np.array_equal(alone.kmers, got[j].kmers)
        assert np.array_equal(alone.counts, got[j].counts)


def test_batch_nul_led_line_ends_its_job(engine):
    W = 10
    a = b"ACGTACGTAC\nCCCCCCCCCC\n\0GGGGGGGGG\nTTTTTTTTTT\n"
    b = b"\0AAAAAAAAA\nGGGGGGGGGG\n"   # NUL first in line 0: just a break there
    got = engine.count_batch([a, b, a], W, 4)
    for j, t in enumerate([a, b, a]):
        keys, counts, nk = pyoracle.count(t, W, 4)
        assert got[j].n_kmers == nk and np.array_equal(got[j].kmers, keys)
        assert np.array_equal(got[j].counts, counts)


def test_batch_waves_under_a_small_budget():
    texts = job_texts(24, seed=3, max_reads=4000)
    with dk.Engine(0, mem_budget=96 << 20) as small:   # 96 MB: forces several waves
        got = small.count_batch(texts, 250, 31, dk.VARIANT_HASH)
        st = small.stats()
    assert st["n_waves"] >= 2
    for j, t in enumerate(texts):
        keys, counts, nk = pyoracle.count(t, 250, 31)
        assert got[j].n_kmers == nk and np.array_equal(got[j].kmers, keys)
        assert np.array_equal(got[j].counts, counts)


def test_batch_many_small_jobs(engine):
    texts = [synth.random_lines(100 + j, 1 + (j % 7), 100) for j in range(300)]
    got = engine.count_batch(texts, 100, 21)
    for j, t in enumerate(texts):
        keys, counts, nk = pyoracle.count(t, 100, 21)
        assert got[j].n_kmers == nk and np.array_equal(got[j].kmers, keys)


@pytest.mark.parametrize("flags", [0, dk.FLAG_STAGE_PAGEABLE])
def test_batch_mixes_pinned_and_pageable_reads(flags):
    """Page-locked jobs go straight to DMA; pageable ones are read in place by
    the device (flags 0, where it can) or go through the staging slots.  No
    pageable copy may overwrite a pinned job's bytes."""
    texts = job_texts(24, seed=7, max_reads=4000)
    pin = [dk.PinnedBuffer(t.size) for t in texts[::2]]
    mixed = []
    for j, t in enumerate(texts):
        if j % 2 == 0:
            b = pin[j // 2]
            b.array[:] = t
            mixed.append(b.array)
        else:
            mixed.append(t)
    with dk.Engine(0, mem_budget=96 << 20, flags=flags) as eng:  # several pipelined waves
        got = eng.count_batch(mixed, 250, 31, dk.VARIANT_HASH)
        st = eng.stats()
    assert st["n_waves"] >= 2
    for j, t in enumerate(texts):
        keys, counts, nk = pyoracle.count(t, 250, 31)
        assert got[j].n_kmers == nk and np.array_equal(got[j].kmers, keys), j
        assert np.array_equal(got[j].counts, counts), j
    for b in pin:
        b.free()


def test_batch_tables_free_while_another_batch_runs():
    """Tables are returned to the pool under their own lock: freeing results of
    one batch while the next runs keeps every table intact."""
    import threading
    texts = job_texts(30, seed=9, max_reads=3000)
    expect = [pyoracle.count(t, 250, 31) for t in texts]
    with dk.Engine(0) as eng:
        first = eng.count_batch_raw(texts[:15], 250, 31, dk.VARIANT_HASH)
        out = {}

        def run_second():
            out["second"] = eng.count_batch(texts[15:], 250, 31, dk.VARIANT_HASH)

        th = threading.Thread(target=run_second)
        th.start()
        for j, t in enumerate(first):                   # free while the second runs
            r = dk.Engine.table_result(t)
            eng.free_table(t)
            keys, counts, nk = expect[j]
            assert r.n_kmers == nk and np.array_equal(r.kmers, keys), j
            assert np.array_equal(r.counts, counts), j
        th.join()
    for j, r in enumerate(out["second"]):
        keys, counts, nk = expect[15 + j]
        assert r.n_kmers == nk and np.array_equal(r.kmers, keys), 15 + j


@pytest.mark.parametrize("variant", [dk.VARIANT_SORT, dk.VARIANT_HASH])
def test_batch_device_resident_tables(engine, variant):
    """With device residency each job's table stays in device memory (no copy
    back) and equals the oracle's; freeing them in any order releases the
    wave's buffer only with its last job."""
    import ctypes
    import torch
    texts = job_texts(24, seed=7)
    outs = engine.count_batch_raw(texts, 250, 31, variant, dk.RESIDENT_DEVICE)
    try:
        for j, t in enumerate(texts):
            keys, counts, nk = pyoracle.count(t, 250, 31)
            o = outs[j]
            assert o.on_device == 1 and int(o.n_kmers) == nk and int(o.n) == keys.size
            n = int(o.n)
            if n == 0:
                continue
            kp = ctypes.cast(o.kmers, ctypes.c_void_p).value
            cp = ctypes.cast(o.counts, ctypes.c_void_p).value

            class _A:
                def __init__(self, p, typestr):
                    self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                                     "data": (p, False), "version": 3}
            gk = torch.as_tensor(_A(kp, "<i8"), device="cuda").cpu().numpy().view(np.uint64)
            gc = torch.as_tensor(_A(cp, "<i4"), device="cuda").cpu().numpy().view(np.uint32)
            assert np.array_equal(gk, keys), j
            assert np.array_equal(gc, counts), j
    finally:
        for o in reversed(outs):
            if o.handle:
                engine.free_table(o)

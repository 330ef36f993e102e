"""Serving loop: continuous batching over engine workers (GPU).

Each served job's table must equal its table when counted alone (and the
oracle's): integer work, exact equality.
"""
import time

import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def texts(n, seed):
    specs = synth.batch_specs(n, seed=seed, median=300, sigma=1.2, cap=3000)
    return [synth.batch_job_text(s, line_width=250) for s in specs]


def test_served_jobs_equal_alone_and_oracle():
    jobs = texts(60, 11)
    with dk.Engine(0) as eng:
        alone = [eng.count(t, 250, 31, dk.VARIANT_HASH) for t in jobs[:10]]
        eng.serve_start(workers=2, max_batch_jobs=64)
        tickets = []
        for i, t in enumerate(jobs):           # bursts arrive while others run
            tickets.append(eng.submit(t, 250, 31, dk.VARIANT_HASH))
            if i % 15 == 14:
                time.sleep(0.01)
        results = [eng.wait(tk, 120_000) for tk in tickets]
        eng.serve_stop()
    batched = 0
    for j, (res, info) in enumerate(results):
        keys, counts, nk = pyoracle.count(jobs[j], 250, 31)
        assert res.n_kmers == nk and np.array_equal(res.kmers, keys), j
        assert np.array_equal(res.counts, counts), j
        if j < 10:
            assert np.array_equal(res.kmers, alone[j].kmers)
            assert np.array_equal(res.counts, alone[j].counts)
        batched += info["batch_jobs"] > 1
        assert info["run_us"] > 0
    assert batched > 0  # jobs were coalesced into batched launches


def test_poll_cancel_and_timeout():
    jobs = texts(8, 12)
    with dk.Engine(0) as eng:
        eng.serve_start(workers=1, max_batch_jobs=2)
        tks = [eng.submit(t, 250, 31) for t in jobs]
        c = eng.cancel(tks[-1])                      # likely still queued
        assert c in (dk.DK_OK, dk.DK_ERR_INVALID_ARG)
        for tk in tks[:-1]:
            res, info = eng.wait(tk, 120_000)
            assert res.n_kmers > 0
        t = dk.Table()
        rc = eng.lib.dk_poll(eng.h, tks[-1], None, None)
        assert rc in (dk.DK_ERR_CANCELLED, dk.DK_OK)
        assert eng.lib.dk_poll(eng.h, 987654321, None, None) == dk.DK_ERR_NOT_FOUND
        eng.serve_stop()


def test_cancelled_running_job_stays_pending_until_its_batch_ends():
    """A job cancelled while its batch runs keeps its text borrowed: it polls
    DK_ERR_PENDING (never a result) until the batch ends, then
    DK_ERR_CANCELLED; the worker then serves the next job normally."""
    big = synth.random_lines(5, 100_000, 250)     # ~25 MB, some ms of work
    small = texts(3, 13)
    with dk.Engine(0) as eng:
        eng.serve_start(workers=1, max_batch_jobs=4)
        tk = eng.submit(big, 250, 31)
        time.sleep(0.02)                           # usually running by now
        assert eng.cancel(tk) in (dk.DK_OK, dk.DK_ERR_INVALID_ARG)
        rc = eng.lib.dk_wait(eng.h, tk, 120_000, None, None)
        assert rc in (dk.DK_ERR_CANCELLED, dk.DK_OK)
        big[:] = 0                                 # the text is no longer read
        for t in small:
            res, _ = eng.wait(eng.submit(t, 250, 31), 120_000)
            keys, counts, nk = pyoracle.count(t, 250, 31)
            assert res.n_kmers == nk and np.array_equal(res.kmers, keys)
            assert np.array_equal(res.counts, counts)
        eng.serve_stop()


def test_wait_on_a_queued_job_returns_when_it_is_cancelled():
    """A thread blocked in dk_wait on a queued job wakes when another thread
    cancels that job, and gets DK_ERR_CANCELLED (not a timeout)."""
    import threading
    big = synth.random_lines(6, 200_000, 250)     # keeps the one worker busy
    queued = texts(1, 14)[0]
    with dk.Engine(0) as eng:
        eng.serve_start(workers=1, max_batch_jobs=1)
        tk_big = eng.submit(big, 250, 31)
        time.sleep(0.02)
        tk = eng.submit(queued, 250, 31)
        out = {}

        def waiter():
            t0 = time.perf_counter()
            out["rc"] = eng.lib.dk_wait(eng.h, tk, 60_000, None, None)
            out["s"] = time.perf_counter() - t0

        th = threading.Thread(target=waiter)
        th.start()
        time.sleep(0.01)
        c = eng.cancel(tk)
        th.join(timeout=30)
        assert not th.is_alive()
        if c == dk.DK_OK:
            assert out["rc"] in (dk.DK_ERR_CANCELLED, dk.DK_OK)
        assert out["s"] < 30
        eng.lib.dk_wait(eng.h, tk_big, 120_000, None, None)
        eng.serve_stop()


def test_serve_stop_releases_results_nobody_took():
    """Finished jobs whose tables were never taken go back to the host pool
    at dk_serve_stop; the context keeps counting afterwards."""
    jobs = texts(4, 15)
    with dk.Engine(0) as eng:
        eng.serve_start(workers=2, max_batch_jobs=4)
        for t in jobs:
            eng.submit(t, 250, 31)
        time.sleep(1.0)   # small jobs: finished by now, their tables not taken
        eng.serve_stop()
        res = eng.count(jobs[0], 250, 31)
        keys, counts, nk = pyoracle.count(jobs[0], 250, 31)
        assert res.n_kmers == nk and np.array_equal(res.kmers, keys)


def test_serve_stop_right_after_start_returns():
    """dk_serve_stop with idle workers (none has slept yet) joins them."""
    with dk.Engine(0) as eng:
        for _ in range(20):
            eng.serve_start(workers=4, max_batch_jobs=4)
            eng.serve_stop()


def test_admission_rejects_oversized_job():
    big = synth.random_lines(1, 200_000, 250)   # ~50 MB of reads, ~44M k-mers
    with dk.Engine(0, mem_budget=256 << 20) as eng:
        eng.serve_start(workers=2, max_batch_jobs=8)
        with pytest.raises(dk.DkError) as e:
            eng.submit(big, 250, 31)
        assert e.value.status == dk.DK_ERR_ADMISSION
        eng.serve_stop()


def test_served_tables_share_the_context_pool_and_outlive_the_server():
    """Host tables of every serving worker come from the context's pool: a
    table handed out by dk_wait stays readable after dk_serve_stop and is
    freed through the context; sizes one worker used are reused by others."""
    import ctypes
    jobs = texts(8, 12)
    with dk.Engine(0) as eng:
        eng.serve_start(workers=2, max_batch_jobs=1)
        held = []
        for t in jobs:
            tk = eng.submit(t, 250, 31, dk.VARIANT_HASH)
            tab, info = dk.Table(), dk.JobInfo()
            assert eng.lib.dk_wait(eng.h, tk, 60_000, ctypes.byref(tab), ctypes.byref(info)) == 0
            held.append(tab)
        eng.serve_stop()
        for j, tab in enumerate(held):
            keys, counts, nk = pyoracle.count(jobs[j], 250, 31)
            n = int(tab.n)
            assert tab.n_kmers == nk and n == keys.size
            assert np.array_equal(np.ctypeslib.as_array(tab.kmers, shape=(n,)), keys), j
            assert np.array_equal(np.ctypeslib.as_array(tab.counts, shape=(n,)), counts), j
            eng.free_table(tab)


def test_served_device_resident_tables():
    """Jobs submitted with device residency get tables left in device memory
    (no copy back), equal to the oracle's; host and device jobs mix."""
    import ctypes
    import torch
    jobs = texts(10, 16)
    with dk.Engine(0) as eng:
        eng.serve_start(workers=2, max_batch_jobs=8)
        tks = [(eng.submit(t, 250, 31, dk.VARIANT_AUTO,
                           dk.RESIDENT_DEVICE if j % 3 else dk.RESIDENT_HOST), j)
               for j, t in enumerate(jobs)]
        for tk, j in tks:
            t, info = eng.wait_raw(tk, 120_000)
            try:
                keys, counts, nk = pyoracle.count(jobs[j], 250, 31)
                assert int(t.n_kmers) == nk and int(t.n) == keys.size
                assert t.on_device == (1 if j % 3 else 0)
                n = int(t.n)
                if n and t.on_device:
                    class _A:
                        def __init__(self, p, typestr):
                            self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                                             "data": (p, False), "version": 3}
                    kp = ctypes.cast(t.kmers, ctypes.c_void_p).value
                    cp = ctypes.cast(t.counts, ctypes.c_void_p).value
                    gk = torch.as_tensor(_A(kp, "<i8"), device="cuda").cpu().numpy().view(np.uint64)
                    gc = torch.as_tensor(_A(cp, "<i4"), device="cuda").cpu().numpy().view(np.uint32)
                elif n:
                    gk = np.ctypeslib.as_array(t.kmers, shape=(n,)).copy()
                    gc = np.ctypeslib.as_array(t.counts, shape=(n,)).copy()
                else:
                    gk, gc = np.zeros(0, np.uint64), np.zeros(0, np.uint32)
                assert np.array_equal(gk, keys) and np.array_equal(gc, counts)
            finally:
                eng.free_table(t)
        eng.serve_stop()

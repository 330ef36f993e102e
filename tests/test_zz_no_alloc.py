"""dk_count_small_noalloc: the count that allocates nothing.

It serves callers that cannot allocate device memory when they need a count
(allocator callbacks, latency-bound serving loops, programs that own all
device memory through their own pool).  Its scratch is one fixed array inside
the library, shared by every call on a device.  This file checks, through the
C ABI, that two calls in a row -- the second on a smaller input, over the
first call's leftovers in that array -- each give exactly dk_count's table,
that several calls queued back to back on one stream do too, and that
oversized inputs are rejected.
The file is named to be collected last; it also passes alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_KMERS = 12288


def _noalloc(lib, text: np.ndarray, W: int, k: int):
    import torch
    nbytes = text.size
    d_text = torch.from_numpy(np.concatenate([text, np.zeros(64, np.uint8)])).cuda()
    lines = (nbytes + 1) // (W + 1) if nbytes else 0
    cap = max(1, lines * max(0, W - k + 1))
    out_k = torch.empty(cap, dtype=torch.int64, device="cuda")
    out_c = torch.empty(cap, dtype=torch.int32, device="cuda")
    summ = torch.full((3,), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.dk_count_small_noalloc(
        ctypes.c_void_p(d_text.data_ptr()), ctypes.c_uint64(nbytes), W, k,
        ctypes.c_void_p(out_k.data_ptr()), ctypes.c_void_p(out_c.data_ptr()),
        ctypes.c_uint64(cap), ctypes.c_void_p(summ.data_ptr()), ctypes.c_void_p(stream))
    if rc != dk.DK_OK:
        return rc, None
    torch.cuda.synchronize()
    s = summ.cpu().numpy()
    nd = int(s[0])
    keys = out_k[:nd].cpu().numpy().view(np.uint64)
    counts = out_c[:nd].cpu().numpy().view(np.uint32)
    return rc, (keys, counts, int(s[1]), int(s[2]))


@pytest.fixture(scope="module")
def lib():
    lib = dk.load_library()
    lib.dk_count_small_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    return lib


def test_noalloc_matches_dk_count_twice(lib, engine):
    g = synth.genome_uniform(41, 5000)
    first = synth.reads(42, g, 100, 120, 150, 150, rc_frac=0.5, err_rate=0.02)   # <= 12,000 k-mers
    second = synth.reads(43, g, 37, 60, 100, 100, rc_frac=0.5, err_rate=0.05)    # smaller, over leftovers
    for text, W, k in ((first, 150, 31), (second, 100, 21)):
        rc, res = _noalloc(lib, text, W, k)
        assert rc == dk.DK_OK
        keys, counts, nk, status = res
        ref = engine.count(text, W, k, dk.VARIANT_SORT)
        assert status == 0
        assert nk == ref.n_kmers
        assert np.array_equal(keys, ref.kmers)
        assert np.array_equal(counts, ref.counts)


def test_noalloc_rejects_oversized_input(lib):
    W, k = 150, 31
    lines = MAX_KMERS // (W - k + 1) + 1
    text = synth.random_lines(3, lines, W)
    rc, _ = _noalloc(lib, text, W, k)
    assert rc == dk.DK_ERR_ADMISSION


def test_noalloc_calls_back_to_back_on_one_stream(lib, engine):
    """Calls queued on one stream run one after the other, each over the
    previous call's leftovers in the shared scratch array: every table equals
    dk_count's."""
    import torch
    g = synth.genome_uniform(51, 5000)
    W, k = 150, 31
    texts = [synth.reads(52 + i, g, 90 - 20 * i, 100, W, W, rc_frac=0.5, err_rate=0.02)
             for i in range(3)]
    stream = torch.cuda.current_stream().cuda_stream
    runs = []
    for text in texts:
        d_text = torch.from_numpy(np.concatenate([text, np.zeros(64, np.uint8)])).cuda()
        lines = (text.size + 1) // (W + 1)
        cap = max(1, lines * (W - k + 1))
        runs.append((text, d_text, cap, torch.empty(cap, dtype=torch.int64, device="cuda"),
                     torch.empty(cap, dtype=torch.int32, device="cuda"),
                     torch.full((3,), -1, dtype=torch.int64, device="cuda")))
    torch.cuda.synchronize()
    for text, d_text, cap, out_k, out_c, summ in runs:
        rc = lib.dk_count_small_noalloc(
            ctypes.c_void_p(d_text.data_ptr()), ctypes.c_uint64(text.size), W, k,
            ctypes.c_void_p(out_k.data_ptr()), ctypes.c_void_p(out_c.data_ptr()),
            ctypes.c_uint64(cap), ctypes.c_void_p(summ.data_ptr()), ctypes.c_void_p(stream))
        assert rc == dk.DK_OK
    torch.cuda.synchronize()
    for text, d_text, cap, out_k, out_c, summ in runs:
        s = summ.cpu().numpy()
        nd = int(s[0])
        ref = engine.count(text, W, k, dk.VARIANT_SORT)
        assert int(s[2]) == 0 and int(s[1]) == ref.n_kmers
        assert np.array_equal(out_k[:nd].cpu().numpy().view(np.uint64), ref.kmers)
        assert np.array_equal(out_c[:nd].cpu().numpy().view(np.uint32), ref.counts)

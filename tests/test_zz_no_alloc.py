"""dk_count_small_noalloc: the count that allocates nothing.

It serves callers that cannot allocate device memory when they need a
count (allocator callbacks, latency-bound serving loops, programs that own all
device memory through their own pool).  Its only scratch is a fixed array in
the library, shared by every call, so this file checks that two calls in a
row -- the second on a smaller input, over the first call's leftovers --
each give exactly dk_count's table, and that oversized inputs are rejected.
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

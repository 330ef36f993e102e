"""The PakMan* k-mer window of the warp-per-line kernels, restated on the CPU.

PakMan*'s k-mer is kmer = ((kmer << 2) | code) & mask over 3-bit codes
(code = (byte >> 1) & 7, Sliding_window, pakman_star/src/kmer_counting.cpp:
313-341).  The warp-per-line kernels (warp_line_kmers<C, 1>) compute it
without a serial roll: each lane packs its C codes' low two bits into one
window and their bit 2 into a second one, a shift-or scan over the 32 lanes
(and a carry over segments of 32*C positions) gives every lane the windows of
the positions before it, and the key at a position is the first window OR'ed
with the second shifted up one slot.  This test walks that scheme lane by
lane for random lines and checks every emitted key against the oracle's
PakMan* walk.  Integer work: exact equality.
"""
import random

import numpy as np
import pytest

from oracle import pyoracle

M64 = (1 << 64) - 1


def _code(b: int) -> int:
    return 0xF0 if b == 10 else (b >> 1) & 7


def _warp_keys(line: bytes, W: int, k: int, C: int):
    """Keys the warp walk emits, by position (None where none ends)."""
    mask = M64 if k == 32 else (1 << (2 * k)) - 1
    B = 2 * C
    out = [None] * W
    carry_w = carry_s = 0
    carry_stop = W
    for seg in range(0, W, 32 * C):
        low, high, first_end = [0] * 32, [0] * 32, [1 << 31] * 32
        for lane in range(32):
            for t in range(C):
                p = seg + lane * C + t
                c = _code(line[p]) if p < W else 0
                end = c == 0xF0
                low[lane] = ((low[lane] << 2) | (0 if end else c & 3)) & M64
                high[lane] = ((high[lane] << 2) | (0 if end else c >> 2)) & M64
                if end and first_end[lane] == 1 << 31:
                    first_end[lane] = p
        stop = min(carry_stop, min(first_end))
        w_inc, s_inc = low[:], high[:]
        o = 1
        while o < 32:  # inclusive shift-or scan over the lanes
            pw, ps = w_inc[:], s_inc[:]
            for lane in range(o, 32):
                if B * o < 64:
                    w_inc[lane] = (w_inc[lane] | (pw[lane - o] << (B * o))) & M64
                    s_inc[lane] = (s_inc[lane] | (ps[lane - o] << (B * o))) & M64
            o <<= 1
        for lane in range(32):
            w_exc = w_inc[lane - 1] if lane else 0
            s_exc = s_inc[lane - 1] if lane else 0
            if B * lane < 64:
                w_exc = (w_exc | (carry_w << (B * lane))) & M64
                s_exc = (s_exc | (carry_s << (B * lane))) & M64
            for t in range(C):
                p = seg + lane * C + t
                up = 2 * (t + 1)
                win = ((w_exc << up) & M64 if up < 64 else 0) | (low[lane] >> (2 * (C - 1 - t)))
                sp = ((s_exc << up) & M64 if up < 64 else 0) | (high[lane] >> (2 * (C - 1 - t)))
                if p < W and p < stop and p >= k - 1:
                    out[p] = (win | ((sp << 2) & M64)) & mask
        carry_w = (((carry_w << (B * 32)) & M64) | w_inc[31]) if B * 32 < 64 else w_inc[31]
        carry_s = (((carry_s << (B * 32)) & M64) | s_inc[31]) if B * 32 < 64 else s_inc[31]
        carry_stop = stop
    return out


@pytest.mark.parametrize("seed", range(6))
def test_warp_window_equals_pakman_walk(seed):
    rng = random.Random(seed)
    for _ in range(12):
        C = rng.choice([1, 2, 4, 5, 8, 16, 32])
        W = rng.randint(1, 600)
        k = rng.randint(1, 32)
        line = bytes(rng.choice(b"ACGTacgtNnRY-\x00") if rng.random() < 0.1 else rng.choice(b"ACGT")
                     for _ in range(W))
        if rng.random() < 0.3:  # a read that ends before the line does
            q = rng.randrange(W)
            line = line[:q] + b"\n" + line[q + 1:]
        keys = [x for x in _warp_keys(line, W, k, C) if x is not None]
        read = line.split(b"\n")[0]
        want = pyoracle.pakman_kmers(b">r\n" + read + b"\n", k)
        assert np.array_equal(np.asarray(keys, dtype=np.uint64), np.asarray(want, dtype=np.uint64)), \
            (seed, C, W, k)

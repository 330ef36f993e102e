"""The k-mer windows of the level-1 scatter (LineWin, DAKC's convention,
k >= 2), restated on the CPU.

The kernel does not roll a key base by base. A chunk's codes are packed two
bits each (C, first code in the top bits) next to the 32 codes before the
chunk (P); the k-mer ending at chunk position q is the bit field
[2(CH-1-q), +2k) of P:C. It is counted when no break byte lies in its window
(break bits of P:C smeared over k positions by doubling shifts) and no stop
('M') came before it (read_till_buf_max, dakc/src/kcounter/kcounter_funcs.cpp:
69-111).  Byte codes enter as the kernel reads them: four per 32-bit word,
0-3 for bases, 0xFF a break, 0xF0 a stop (bit 7 marks both, bit 0 tells them
apart).  This test walks that scheme for random lines, both chunk widths, and
checks the table against the oracle's.  Integer work: exact equality.
"""
import random

import numpy as np
import pytest

from oracle import pyoracle

M64 = (1 << 64) - 1
CODE = {ord("C"): 0, ord("A"): 1, ord("T"): 2, ord("G"): 3, ord("M"): 0xF0}


def _pack4(w):  # four byte codes -> eight bits, first code on top
    x = w & 0x03030303
    return (((x & 3) << 6) | ((x >> 4) & 0x30) | ((x >> 14) & 0x0C) | (x >> 24)) & 0xFF


def _flags4(m):  # bit 7 of byte u -> bit u
    return ((((m >> 7) & 0x01010101) * 0x00204081) >> 21) & 0xF


def _pack(codes, CH):
    c = brk = stp = 0
    for g in range(CH // 4):
        w = sum(codes[4 * g + u] << (8 * u) for u in range(4))
        c |= _pack4(w) << (2 * CH - 8 - 8 * g)
        brk |= _flags4(w & 0x80808080) << (4 * g)
        stp |= _flags4(w & ~(w << 7) & 0x80808080 & 0xFFFFFFFF) << (4 * g)
    return c & M64, brk, stp


def _window_keys(line: bytes, k: int, CH: int):
    W = len(line)
    codes = [CODE.get(b, 0xFF) for b in line]
    kmask = M64 >> (64 - 2 * k)
    warm = min(k - 1, W)
    P, B, t = _pack([0xFF if warm - 32 + i < 0 else codes[warm - 32 + i] for i in range(32)], 32)
    stopped = t != 0
    out = []
    for p0 in range(warm, W, CH):
        n = min(W - p0, CH)
        C, brk, stp = _pack([codes[p0 + q] if q < n else 0xF0 for q in range(CH)], CH)
        m = ((brk << 32) | B) & M64
        sm, w = m, 1
        while 2 * w <= k:
            sm = (sm | (sm << w)) & M64
            w <<= 1
        if w < k:
            sm = (sm | (sm << (k - w))) & M64
        v = (~(sm >> 32)) & 0xFFFFFFFF
        if CH < 32:
            v &= (1 << CH) - 1
        if stopped:
            v = 0
        if stp:
            v &= (1 << ((stp & -stp).bit_length() - 1)) - 1
        lo = C if CH == 32 else (((P << (2 * CH)) | C) & M64)
        hi = P if CH == 32 else (P >> (64 - 2 * CH))
        for q in range(CH):
            if (v >> q) & 1:
                s = 2 * (CH - 1 - q)
                x = lo if s == 0 else (((lo >> s) | (hi << (64 - s))) & M64)
                out.append(x & kmask)
        P = lo
        B = (m >> CH) & 0xFFFFFFFF
        stopped = stopped or stp != 0
    return out


@pytest.mark.parametrize("seed", range(8))
def test_windows_equal_oracle_table(seed):
    rng = random.Random(seed)
    for _ in range(40):
        W = rng.choice([2, 5, 20, 31, 32, 33, 40, 63, 64, 100, 150, 151, 250, 256])
        k = rng.randint(2, 32)
        p_break = rng.choice([0.0, 0.01, 0.05, 0.3])
        p_stop = rng.choice([0.0, 0.0, 0.005, 0.05])
        line = bytes(ord("M") if (r := rng.random()) < p_stop else
                     (ord("N") if r < p_stop + p_break else rng.choice(b"ACGT")) for _ in range(W))
        keys, counts, nk = pyoracle.count(np.frombuffer(line + b"\n", np.uint8), W, k)
        for CH in (16, 32):
            got = np.asarray(_window_keys(line, k, CH), dtype=np.uint64)
            gk, gc = np.unique(got, return_counts=True)
            assert got.size == nk and np.array_equal(gk, keys) and np.array_equal(gc, counts), \
                (seed, W, k, CH)

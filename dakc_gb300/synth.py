"""Seeded synthetic workloads in DAKC's fixed-width read format.

The generator itself is C++ (``synth/dk_synth.cpp``): output depends only on the
seed and parameters, on any machine and for any thread count.  This module
wraps it and defines the benchmark workloads by their shapes:

* ``plain_1m``   -- 1 Mbp iid genome, 100,000 reads x 150 bp, 50/50 strand,
  0.1% substitutions, k=31 (the CPU-runnable plain count).
* ``large_100m`` -- 100 Mbp genome, 20% of it in 200 repeat families
  (1-5 kbp, 10-100 copies, 2% divergence), 30x coverage of 150 bp reads
  (20M reads, 3 Gbases), 1% substitutions, 50/50 strand, k=31.
* ``zipf_skew``  -- 10M reads x 150 bp over a 50 Mbp background; 70% of reads
  copy one of 1,000 hot templates drawn Zipf(s=1.1), which makes the top
  1,000 k-mers each occur >= 10^5 times (asserted), k in {17, 21, 31}.
* ``batch_jobs`` -- independent read sets with lognormal read counts
  (median 20,000, sigma 1.5, cap 5M), read lengths U[100, 250] padded with
  'M' to 250, per-job 0.5-5 Mbp genomes, 0.5% substitutions.

The reference's own generator is unseeded and its reads come from ART
(syngen/inputgenerator.cpp:15-19, syngen/synthetic_generator.sh:11); these
seeded stand-ins reproduce the shapes, not the bytes.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "synth", "_build", "libdk_synth.so")
_lib = None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        from . import build as _b
        _b.build_synth()
    lib = ctypes.CDLL(_LIB_PATH)
    u64, i32, f64, vp = ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    lib.dks_genome_uniform.argtypes = [u64, u64, vp, i32]
    lib.dks_genome_repeats.argtypes = [u64, u64, i32, i32, i32, i32, i32, f64, f64, vp, i32]
    lib.dks_genome_repeats.restype = u64
    lib.dks_reads.argtypes = [u64, vp, u64, u64, i32, i32, i32, f64, f64, vp, i32]
    lib.dks_zipf_reads.argtypes = [u64, vp, u64, u64, i32, f64, i32, f64, f64, vp, vp, i32]
    lib.dks_lognormal_counts.argtypes = [u64, i32, f64, f64, u64, u64, vp]
    lib.dks_uniform.argtypes = [u64, u64, f64, f64, vp]
    lib.dks_exponential.argtypes = [u64, u64, f64, vp]
    lib.dks_log.argtypes = [f64]
    lib.dks_log.restype = f64
    lib.dks_exp.argtypes = [f64]
    lib.dks_exp.restype = f64
    _lib = lib
    return lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def genome_uniform(seed: int, length: int, threads: int = 0) -> np.ndarray:
    out = np.empty(length, dtype=np.uint8)
    _load().dks_genome_uniform(seed, length, _ptr(out), threads)
    return out


def genome_repeats(seed: int, length: int, nfam: int = 200, lmin: int = 1000, lmax: int = 5000,
                   cmin: int = 10, cmax: int = 100, repeat_frac: float = 0.2, div: float = 0.02,
                   threads: int = 0) -> tuple[np.ndarray, int]:
    out = np.empty(length, dtype=np.uint8)
    rep = _load().dks_genome_repeats(seed, length, nfam, lmin, lmax, cmin, cmax, repeat_frac, div,
                                     _ptr(out), threads)
    return out, int(rep)


def reads(seed: int, genome: np.ndarray, nreads: int, len_min: int, len_max: int, line_width: int,
          rc_frac: float = 0.5, err_rate: float = 0.0, threads: int = 0) -> np.ndarray:
    if len_max > line_width or len_max > genome.size or len_min < 1 or len_min > len_max:
        raise ValueError("bad read length range")
    out = np.empty(nreads * (line_width + 1), dtype=np.uint8)
    _load().dks_reads(seed, _ptr(genome), genome.size, nreads, len_min, len_max, line_width,
                      rc_frac, err_rate, _ptr(out), threads)
    return out


def zipf_reads(seed: int, background: np.ndarray, nreads: int, read_len: int, hot_frac: float,
               ntemplates: int, s: float, err_rate: float = 0.0, threads: int = 0
               ) -> tuple[np.ndarray, np.ndarray]:
    out = np.empty(nreads * (read_len + 1), dtype=np.uint8)
    hot = np.zeros(ntemplates, dtype=np.uint64)
    _load().dks_zipf_reads(seed, _ptr(background), background.size, nreads, read_len, hot_frac,
                           ntemplates, s, err_rate, _ptr(out), _ptr(hot), threads)
    return out, hot


def lognormal_counts(seed: int, n: int, median: float, sigma: float, lo: int, cap: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint64)
    _load().dks_lognormal_counts(seed, n, median, sigma, lo, cap, _ptr(out))
    return out


def uniform(seed: int, n: int, lo: float, hi: float) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    _load().dks_uniform(seed, n, lo, hi, _ptr(out))
    return out


def exponential(seed: int, n: int, rate: float) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    _load().dks_exponential(seed, n, rate, _ptr(out))
    return out


# --------------------------------------------------------------- workloads
@dataclass
class ReadSet:
    """Reads in DAKC text format plus the counting parameters."""
    name: str
    text: np.ndarray      # uint8, n_lines * (line_width + 1) bytes
    line_width: int
    k: int
    seed: int

    @property
    def n_lines(self) -> int:
        return self.text.size // (self.line_width + 1)


def plain_1m(seed: int = 1, k: int = 31) -> ReadSet:
    g = genome_uniform(seed, 1_000_000)
    t = reads(seed + 1, g, 100_000, 150, 150, 150, rc_frac=0.5, err_rate=0.001)
    return ReadSet("plain_1m", t, 150, k, seed)


def large_100m(seed: int = 2, k: int = 31, genome_len: int = 100_000_000, coverage: float = 30.0
               ) -> ReadSet:
    g, _ = genome_repeats(seed, genome_len)
    n = int(round(coverage * genome_len / 150))
    t = reads(seed + 1, g, n, 150, 150, 150, rc_frac=0.5, err_rate=0.01)
    return ReadSet("large_100m", t, 150, k, seed)


ZIPF_HOT_FRAC = 0.7
ZIPF_TEMPLATES = 1000
ZIPF_S = 1.1


def zipf_skew(seed: int = 3, k: int = 31, nreads: int = 10_000_000, background_len: int = 50_000_000,
              check: bool = True) -> ReadSet:
    bg = genome_uniform(seed, background_len)
    t, hot = zipf_reads(seed + 1, bg, nreads, 150, ZIPF_HOT_FRAC, ZIPF_TEMPLATES, ZIPF_S,
                        err_rate=0.001)
    if check and nreads >= 10_000_000:
        # templates 0..8 carry 9 x (150-k+1) >= 1,000 distinct k-mers for k <= 31; each of
        # their k-mers occurs at least as often as its template is copied
        assert int(hot[:9].min()) >= 100_000, hot[:9]
    return ReadSet(f"zipf_skew_k{k}", t, 150, k, seed)


@dataclass
class JobSpec:
    job_id: int
    seed: int
    genome_len: int
    n_reads: int


def batch_specs(njobs: int = 4096, seed: int = 4, median: float = 20_000, sigma: float = 1.5,
                cap: int = 5_000_000) -> list[JobSpec]:
    counts = lognormal_counts(seed, njobs, median, sigma, 1, cap)
    glens = uniform(seed + 1, njobs, 500_000, 5_000_001)
    return [JobSpec(j, seed * 1_000_003 + j, int(glens[j]), int(counts[j])) for j in range(njobs)]


def batch_job_text(spec: JobSpec, line_width: int = 250, len_min: int = 100, len_max: int = 250,
                   err_rate: float = 0.005, max_reads: int | None = None) -> np.ndarray:
    g = genome_uniform(spec.seed, spec.genome_len, threads=1)
    n = spec.n_reads if max_reads is None else min(spec.n_reads, max_reads)
    return reads(spec.seed + 7, g, n, len_min, len_max, line_width, rc_frac=0.5,
                 err_rate=err_rate, threads=1)


def random_lines(seed: int, n_lines: int, line_width: int, alphabet: bytes = b"ACGT") -> np.ndarray:
    """Lines of iid symbols from `alphabet` (for edge-case tests)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = np.frombuffer(alphabet, dtype=np.uint8)
    body = a[rng.integers(0, a.size, size=(n_lines, line_width))]
    out = np.empty((n_lines, line_width + 1), dtype=np.uint8)
    out[:, :line_width] = body
    out[:, line_width] = ord("\n")
    return out.reshape(-1)

"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only the tests, the smoke check and the benchmark's CPU-baseline leg import
this module, and only as the checker / the timed CPU baseline; the engine
never calls it.

* ``count``      -- dk_oracle.c's single-threaded restatement (extract, LSD
                    radix sort, run-length), the parity checker.
* ``count_mt``   -- the same table on T host threads (key ranges sorted and
                    run-length reduced independently), the checker for inputs
                    of billions of k-mers.
* ``dakc_port``  -- DAKC's two phases on P host threads (owner hash
                    MurmurHash64A % P, per-owner sort + run-length), timed as
                    the CPU baseline.
* ``ref_table``  -- runs the reference's own kcounter sources, compiled
                    unmodified against the shim (oracle/_ref), on P forked PEs.
                    Only available where the reference tree was present to
                    compile them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libdk_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_TREE = "/root/reference"


class _Table(ctypes.Structure):
    _fields_ = [("kmers", ctypes.POINTER(ctypes.c_uint64)),
                ("counts", ctypes.POINTER(ctypes.c_uint32)),
                ("n", ctypes.c_uint64),
                ("n_kmers", ctypes.c_uint64)]


_lib = None


def build_lib() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build_lib()
        lib = ctypes.CDLL(LIB)
        vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        lib.dko_count.argtypes = [vp, u64, i32, i32, ctypes.POINTER(_Table)]
        lib.dko_count_mt.argtypes = [vp, u64, i32, i32, i32, ctypes.POINTER(_Table)]
        lib.dko_dakc_port.argtypes = [vp, u64, i32, i32, i32, i32, ctypes.POINTER(_Table),
                                      ctypes.POINTER(ctypes.c_double)]
        lib.dko_free.argtypes = [ctypes.POINTER(_Table)]
        lib.dko_num_lines.argtypes = [vp, u64, i32]
        lib.dko_num_lines.restype = ctypes.c_int64
        lib.dko_murmur64a.argtypes = [u64, u64]
        lib.dko_murmur64a.restype = u64
        lib.dko_code_table.restype = ctypes.POINTER(ctypes.c_uint8)
        _lib = lib
    return _lib


class OracleError(RuntimeError):
    pass


def _as_bytes(text) -> np.ndarray:
    if isinstance(text, (bytes, bytearray)):
        return np.frombuffer(bytes(text), dtype=np.uint8)
    return np.ascontiguousarray(text, dtype=np.uint8)


def _take(t: _Table):
    n = int(t.n)
    if n:
        keys = np.ctypeslib.as_array(t.kmers, shape=(n,)).copy()
        counts = np.ctypeslib.as_array(t.counts, shape=(n,)).copy()
    else:
        keys = np.zeros(0, np.uint64)
        counts = np.zeros(0, np.uint32)
    return keys, counts, int(t.n_kmers)


def count(text, line_width: int, k: int):
    """(keys uint64 sorted, counts uint32, n_kmers) by the single-threaded restatement."""
    buf = _as_bytes(text)
    lib = _load()
    t = _Table()
    rc = lib.dko_count(buf.ctypes.data, buf.size, line_width, k, ctypes.byref(t))
    try:
        if rc == -1:
            raise OracleError("invalid arguments")
        out = _take(t)
        if rc == -2:
            raise OracleError("count overflows 32 bits")
        return out
    finally:
        lib.dko_free(ctypes.byref(t))


def count_mt(text, line_width: int, k: int, threads: int = 0):
    """(keys, counts, n_kmers) of ``count`` on `threads` host threads (0 = all)."""
    buf = _as_bytes(text)
    lib = _load()
    t = _Table()
    rc = lib.dko_count_mt(buf.ctypes.data, buf.size, line_width, k, threads, ctypes.byref(t))
    try:
        if rc == -1:
            raise OracleError("invalid arguments or out of host memory")
        out = _take(t)
        if rc == -2:
            raise OracleError("count overflows 32 bits")
        return out
    finally:
        lib.dko_free(ctypes.byref(t))


def dakc_port(text, line_width: int, k: int, pes: int, merge: bool = True):
    """Run the P-thread DAKC port; returns ((keys, counts, n_kmers) or None, seconds)."""
    buf = _as_bytes(text)
    lib = _load()
    t = _Table()
    secs = ctypes.c_double(0)
    rc = lib.dko_dakc_port(buf.ctypes.data, buf.size, line_width, k, pes, 1 if merge else 0,
                           ctypes.byref(t), ctypes.byref(secs))
    try:
        if rc == -1:
            raise OracleError("invalid arguments")
        if merge:
            return _take(t), secs.value
        return (None, None, int(t.n_kmers)), secs.value
    finally:
        lib.dko_free(ctypes.byref(t))


def num_lines(text, line_width: int) -> int:
    buf = _as_bytes(text)
    return int(_load().dko_num_lines(buf.ctypes.data, buf.size, line_width))


def murmur64a(key: int, seed: int = 0x9E3779B97F4A7C15) -> int:
    return int(_load().dko_murmur64a(key, seed))


def code_table() -> np.ndarray:
    p = _load().dko_code_table()
    return np.ctypeslib.as_array(p, shape=(256,)).copy()


# ------------------------------------------------------- reference (shim)
def ref_binary(k: int, line_width: int, hitter: int = 0, build: bool = True) -> str | None:
    """Path of the shim-built reference binary for (k, READLEN, HITTER), building it
    from the reference tree when that tree is present; None when unavailable."""
    path = os.path.join(REF_DIR, f"dakc_ref_k{k}_r{line_width}_h{hitter}")
    if os.path.exists(path):
        return path
    if not build or not os.path.isdir(os.path.join(REFERENCE_TREE, "dakc", "src")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"K={k}", f"R={line_width}", f"H={hitter}",
                    f"REF={REFERENCE_TREE}"], check=True)
    return path


def read_table_file(path: str):
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:4] != b"DKT1":
        raise OracleError("bad table file")
    n = int(np.frombuffer(raw, np.uint64, 1, 4)[0])
    nk = int(np.frombuffer(raw, np.uint64, 1, 12)[0])
    keys = np.frombuffer(raw, np.uint64, n, 20).copy()
    counts = np.frombuffer(raw, np.uint32, n, 20 + 8 * n).copy()
    return keys, counts, nk


def ref_table(text, line_width: int, k: int, pes: int = 1, hitter: int = 0, timeout: float = 600):
    """Run the reference's own counting code on `pes` forked PEs.

    Returns ((keys, counts, n_kmers), stdout).  Raises OracleError when the
    binary is unavailable or when the reference's behaviour is undefined for
    this input (a PE that receives no k-mer)."""
    exe = ref_binary(k, line_width, hitter)
    if exe is None:
        raise OracleError("reference binary unavailable (reference tree absent)")
    buf = _as_bytes(text)
    with tempfile.TemporaryDirectory() as d:
        inp = os.path.join(d, "reads.txt")
        out = os.path.join(d, "table.bin")
        buf.tofile(inp)
        p = subprocess.run([exe, inp, str(pes), out], capture_output=True, text=True, timeout=timeout)
        if p.returncode != 0:
            raise OracleError(f"reference exited {p.returncode}: {p.stderr.strip()[:200]}")
        return read_table_file(out), p.stdout


def pakman_binary(k: int, build: bool = True) -> str | None:
    """Path of PakMan*'s k-mer counting built against the one-rank MPI
    stand-in (oracle/_ref/pakman_ref_k<k>); None when unavailable."""
    path = os.path.join(REF_DIR, f"pakman_ref_k{k}")
    if os.path.exists(path):
        return path
    if not build or not os.path.isdir(os.path.join(REFERENCE_TREE, "pakman_star", "src")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "pakman", f"K={k}", f"REF={REFERENCE_TREE}"],
                   check=True)
    return path


def pakman_ref_table(fasta, k: int, batch: int = 100_000_000, timeout: float = 600):
    """Run PakMan*'s own k-mer counting (one rank) on a FASTA buffer; returns
    (keys, counts) sorted by k-mer."""
    exe = pakman_binary(k)
    if exe is None:
        raise OracleError("PakMan* binary unavailable (reference tree absent)")
    buf = _as_bytes(fasta)
    with tempfile.TemporaryDirectory() as d:
        inp = os.path.join(d, "reads.fa")
        out = os.path.join(d, "table.bin")
        buf.tofile(inp)
        p = subprocess.run([exe, inp, str(batch), out], capture_output=True, text=True,
                           timeout=timeout)
        if p.returncode != 0:
            raise OracleError(f"PakMan* exited {p.returncode}: {p.stderr.strip()[:200]}")
        with open(out, "rb") as f:
            raw = f.read()
    if raw[:4] != b"PKT1":
        raise OracleError("bad table file")
    n = int(np.frombuffer(raw, np.uint64, 1, 4)[0])
    rec = np.frombuffer(raw, dtype=np.dtype([("k", "<u8"), ("c", "<u4")]), count=n, offset=12)
    return rec["k"].copy(), rec["c"].copy()


def pakman_histogram_cutoff(counts, num_buckets: int):
    """PakMan*'s count histogram and min-bucket cut-off, restated from
    pakman_star/src/kmer_histogram.cpp:72-130: hist[c] = distinct k-mers with
    count c < num_buckets; min_bucket = the first minimum over hist[1:]
    (std::min_element, :109-110), 0 when num_buckets == 0; the kept k-mers are
    those with count >= min_bucket (:123-130)."""
    counts = np.asarray(counts, dtype=np.uint64)
    if num_buckets <= 0:
        return np.zeros(0, np.uint64), 0
    hist = np.zeros(num_buckets, np.uint64)
    small = counts[counts < num_buckets].astype(np.int64)
    if small.size:
        hist += np.bincount(small, minlength=num_buckets).astype(np.uint64)[:num_buckets]
    if num_buckets == 1:
        return hist, 0
    return hist, 1 + int(np.argmin(hist[1:]))


def fq2txt(fastq: bytes) -> tuple[bytes, int]:
    """syngen/fq2txtmaker.sh:12-18 restated: keep lines NR%4==2 (the reads of
    4-line FASTQ records), pad each with spaces to the longest (printf
    "%-Ns"), then turn every space into 'M' (sed 's/ /M/g').  Returns the
    DAKC text and its line width."""
    lines = fastq.split(b"\n")
    if fastq.endswith(b"\n"):
        lines = lines[:-1]
    seqs = lines[1::4]
    if not seqs:
        return b"", 0
    w = max(len(s) for s in seqs)
    return b"".join(s.ljust(w, b" ").replace(b" ", b"M") + b"\n" for s in seqs), w


def pakman_kmers(buf: bytes, k: int) -> np.ndarray:
    """PakMan*'s k-mer walk over a FASTA buffer, restated from
    Sliding_window, pakman_star/src/kmer_counting.cpp:283-341: start at the
    first '>'; repeatedly skip a line (the header), then roll the next line
    with kmer = ((kmer << 2) | ((byte >> 1) & 7)) & mask (char_to_el /
    kmer_shift, pakman_star/includes/distribute_kmers.h), emitting a k-mer at
    every byte from the k-th on; stop when fewer than k bytes remain after a
    header (:301).  Pure Python: small inputs only."""
    mask = (1 << (2 * k)) - 1
    L = len(buf)
    p = buf.find(b">")
    if p < 0:
        return np.zeros(0, np.uint64)
    out = []
    nl = 10
    while p < L:
        while p < L and buf[p] != nl:
            p += 1
        p += 1
        if p + k > L:
            break
        kmer = 0
        i = 0
        while p < L and buf[p] != nl and i < k - 1:
            kmer = ((kmer << 2) | ((buf[p] >> 1) & 7)) & mask
            p += 1
            i += 1
        while p < L and buf[p] != nl:
            kmer = ((kmer << 2) | ((buf[p] >> 1) & 7)) & mask
            p += 1
            out.append(kmer)
        p += 1
    return np.array(out, dtype=np.uint64)


def table_of(kmers: np.ndarray):
    """(sorted distinct k-mers, their counts as uint32, occurrences)."""
    keys, counts = np.unique(np.asarray(kmers, dtype=np.uint64), return_counts=True)
    return keys, counts.astype(np.uint32), int(np.asarray(kmers).size)


def format_lines(text: bytes, fmt: str) -> list[bytes]:
    """The reads of `text` in layout fmt ('lines', 'fastq', 'fasta'): the
    bytes of each read line (FASTQ line 2 of each record, fq2txtmaker.sh:12;
    FASTA: from the line holding the first '>', every second line,
    kmer_counting.cpp:288-300)."""
    lines = text.split(b"\n")
    if text.endswith(b"\n"):
        lines = lines[:-1]
    if fmt == "lines":
        return lines
    if fmt == "fastq":
        return lines[1::4]
    g = text.find(b">")
    if g < 0:
        return []
    h = text[:g].count(b"\n")
    return lines[h + 1::2]

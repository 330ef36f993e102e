"""dakc_gb300 -- GB300-native k-mer counting, a drop-in for DAKC's counting path.

The engine is native code (``_build/libdakc_gb300.so``: sm_103a CUDA kernels
and a C++ host pipeline behind the C ABI of ``include/dakc_gb300.h``).  This
module is a thin ctypes mirror of that ABI for Python callers, tests and the
benchmark.  There is no CPU fallback: loading fails loudly when the library
is missing, and counting fails with ``DkError`` when no GPU is usable.

DAKC's counter is ``kmercounter(read_chunk, vectordbg)``
(dakc/src/kcounter/kcounter.hpp:84-99): k and the line width are compile-time
there (KMERLEN, READLEN) and the table is left in the member ``lightdbg``.
``Engine.count(text, line_width, k)`` takes the same read buffer and returns
the same table, globally sorted: ``(kmers uint64[n], counts uint32[n],
n_kmers)``.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdakc_gb300.so")

DK_OK = 0
DK_ERR_INVALID_ARG = -1
DK_ERR_OOM = -2
DK_ERR_COUNT_OVERFLOW = -3
DK_ERR_CUDA = -4
DK_ERR_TIMEOUT = -5
DK_ERR_ADMISSION = -6
DK_ERR_PENDING = -7
DK_ERR_NOT_FOUND = -8
DK_ERR_CANCELLED = -9
DK_ERR_NO_DEVICE = -10

VARIANT_AUTO, VARIANT_SORT, VARIANT_HASH = 0, 1, 2
CONV_DAKC, CONV_PAKMAN = 0, 1
FLAG_STREAM_ALL = 1  # dk_config.flags: copy every host table out group by group
FLAG_STAGE_PAGEABLE = 2  # dk_config.flags: stage pageable reads through page-locked slots
FLAG_NO_GRAPH = 4  # dk_config.flags: batch waves without the CUDA graph
FLAG_GRAPH_MIN_BUFFERS = 8  # dk_config.flags: wave graphs at minimal buffers (fallback tests)

FORMAT_LINES, FORMAT_FASTQ, FORMAT_FASTA = 0, 1, 2
RESIDENT_HOST, RESIDENT_DEVICE = 0, 1

# exported symbols, in the order include/dakc_gb300.h declares them
ABI_SYMBOLS = [
    "dk_create", "dk_destroy", "dk_strerror", "dk_last_error_string", "dk_abi_version",
    "dk_count", "dk_count_device", "dk_table_free", "dk_last_stats", "dk_num_lines",
    "dk_host_alloc", "dk_host_free", "dk_count_small_noalloc", "dk_count_batch",
    "dk_serve_start", "dk_submit", "dk_poll", "dk_wait", "dk_cancel", "dk_serve_stop",
    "dk_autotune", "dk_autotune_reset",
    "dk_table_histogram", "dk_table_filter", "dk_table_lookup", "dk_table_pairs",
    "dk_count_format",
]


class DkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("reserved0", ctypes.c_int),
                ("mem_budget", ctypes.c_uint64), ("flags", ctypes.c_uint64)]


class InputDesc(ctypes.Structure):
    _fields_ = [("line_width", ctypes.c_int), ("k", ctypes.c_int), ("convention", ctypes.c_int),
                ("variant", ctypes.c_int), ("residency", ctypes.c_int),
                ("l1_bits", ctypes.c_int), ("bin_target", ctypes.c_int),
                ("reserved", ctypes.c_int)]


class Table(ctypes.Structure):
    _fields_ = [("kmers", ctypes.POINTER(ctypes.c_uint64)),
                ("counts", ctypes.POINTER(ctypes.c_uint32)),
                ("n", ctypes.c_uint64), ("n_kmers", ctypes.c_uint64),
                ("on_device", ctypes.c_int), ("variant_used", ctypes.c_int),
                ("handle", ctypes.c_uint64)]


class Job(ctypes.Structure):
    _fields_ = [("text", ctypes.c_void_p), ("nbytes", ctypes.c_uint64)]


class JobInfo(ctypes.Structure):
    _fields_ = [("queued_us", ctypes.c_double), ("run_us", ctypes.c_double),
                ("batch_jobs", ctypes.c_int), ("worker", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("ms_device", ctypes.c_double), ("ms_h2d", ctypes.c_double),
                ("ms_d2h", ctypes.c_double), ("ms_wall", ctypes.c_double),
                ("ms_stage", ctypes.c_double * 8),
                ("n_kmers", ctypes.c_uint64), ("n_distinct", ctypes.c_uint64),
                ("n_lines", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("dev_bytes_peak", ctypes.c_uint64), ("variant_used", ctypes.c_int),
                ("partition_levels", ctypes.c_int), ("n_bins", ctypes.c_uint64),
                ("ms_kernel", ctypes.c_double * 8), ("launches_kernel", ctypes.c_uint64 * 8),
                ("n_partitioned", ctypes.c_uint64), ("n_waves", ctypes.c_uint64),
                ("n_bins_resorted", ctypes.c_uint64), ("n_bins_big", ctypes.c_uint64),
                ("n_bins_retried", ctypes.c_uint64), ("n_groups", ctypes.c_uint64),
                ("table_streamed", ctypes.c_uint64), ("upload_chunks", ctypes.c_uint64),
                ("n_bins_packed", ctypes.c_uint64), ("n_bins_fallback", ctypes.c_uint64),
                ("upload_in_place", ctypes.c_uint64), ("graph_waves", ctypes.c_uint64),
                ("graph_builds", ctypes.c_uint64), ("graph_retries", ctypes.c_uint64)]

    KERNEL_NAMES = ["extract_count", "extract_scatter", "partition_hist", "partition_scatter",
                    "bin_count", "compact", "wave_graph", "other"]

    def as_dict(self) -> dict:
        arrays = ("ms_stage", "ms_kernel", "launches_kernel")
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in arrays}
        for a in arrays:
            d[a] = list(getattr(self, a))
        return d


class Tune(ctypes.Structure):
    _fields_ = [("l1_bits", ctypes.c_int), ("bin_target", ctypes.c_int), ("variant", ctypes.c_int),
                ("candidates", ctypes.c_int), ("ms_device", ctypes.c_double),
                ("ms_auto", ctypes.c_double)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the engine library (build it first if it is absent and nvcc exists).
    DAKC_GB300_LIB, when set, names another build of the library to load."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("DAKC_GB300_LIB", path)
    if not os.path.exists(path):
        from . import build as _b
        _b.build_engine()
    lib = ctypes.CDLL(path)
    vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
    lib.dk_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
    lib.dk_destroy.argtypes = [vp]
    lib.dk_strerror.argtypes = [i32]
    lib.dk_strerror.restype = ctypes.c_char_p
    lib.dk_last_error_string.argtypes = [vp]
    lib.dk_last_error_string.restype = ctypes.c_char_p
    lib.dk_count.argtypes = [vp, vp, u64, ctypes.POINTER(InputDesc), ctypes.POINTER(Table)]
    lib.dk_count_device.argtypes = [vp, vp, u64, ctypes.POINTER(InputDesc), ctypes.POINTER(Table)]
    lib.dk_table_free.argtypes = [vp, ctypes.POINTER(Table)]
    lib.dk_last_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.dk_autotune.argtypes = [vp, vp, u64, ctypes.POINTER(InputDesc), ctypes.POINTER(Tune)]
    lib.dk_autotune_reset.argtypes = [vp]
    lib.dk_table_histogram.argtypes = [vp, ctypes.POINTER(Table), ctypes.c_uint32, vp,
                                       ctypes.POINTER(ctypes.c_uint32)]
    lib.dk_table_filter.argtypes = [vp, ctypes.POINTER(Table), ctypes.c_uint32, ctypes.POINTER(Table)]
    lib.dk_table_lookup.argtypes = [vp, ctypes.POINTER(Table), vp, u64, vp]
    lib.dk_table_pairs.argtypes = [vp, ctypes.POINTER(Table), vp]
    lib.dk_count_format.argtypes = [vp, vp, u64, i32, ctypes.POINTER(InputDesc),
                                    ctypes.POINTER(Table), ctypes.POINTER(ctypes.c_int)]
    lib.dk_num_lines.argtypes = [vp, u64, i32]
    lib.dk_num_lines.restype = ctypes.c_int64
    lib.dk_count_batch.argtypes = [vp, ctypes.POINTER(Job), i32, ctypes.POINTER(InputDesc),
                                   ctypes.POINTER(Table)]
    lib.dk_serve_start.argtypes = [vp, i32, i32]
    lib.dk_submit.argtypes = [vp, vp, u64, ctypes.POINTER(InputDesc), ctypes.POINTER(u64)]
    lib.dk_poll.argtypes = [vp, u64, ctypes.POINTER(Table), ctypes.POINTER(JobInfo)]
    lib.dk_wait.argtypes = [vp, u64, i32, ctypes.POINTER(Table), ctypes.POINTER(JobInfo)]
    lib.dk_cancel.argtypes = [vp, u64]
    lib.dk_serve_stop.argtypes = [vp]
    lib.dk_host_alloc.argtypes = [u64, ctypes.POINTER(vp)]
    lib.dk_host_free.argtypes = [vp]
    _lib = lib
    return lib


def _buf_ptr(text) -> tuple[int, int, object]:
    if isinstance(text, (bytes, bytearray)):
        arr = np.frombuffer(bytes(text), dtype=np.uint8)
    else:
        arr = np.ascontiguousarray(text, dtype=np.uint8)
    return arr.ctypes.data, arr.size, arr


@dataclass
class CountResult:
    kmers: np.ndarray   # uint64, ascending
    counts: np.ndarray  # uint32
    n_kmers: int
    variant: int


class PinnedBuffer:
    """Page-locked host bytes from the engine (cudaMallocHost); numpy view in .array."""

    def __init__(self, nbytes: int):
        lib = load_library()
        p = ctypes.c_void_p()
        rc = lib.dk_host_alloc(max(1, nbytes), ctypes.byref(p))
        if rc != DK_OK:
            raise DkError(rc, "dk_host_alloc failed")
        self._p = p
        self.nbytes = nbytes
        buf = (ctypes.c_uint8 * max(1, nbytes)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.uint8, count=nbytes)

    @property
    def ptr(self) -> int:
        return self._p.value

    def free(self):
        if self._p:
            load_library().dk_host_free(self._p)
            self._p = None
            self.array = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Engine:
    """One engine context: a CUDA stream, its device arenas and table pool."""

    def __init__(self, device: int = 0, mem_budget: int = 0, flags: int = 0):
        self.lib = load_library()
        cfg = Config(device, 0, mem_budget, flags)
        h = ctypes.c_void_p()
        rc = self.lib.dk_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != DK_OK:
            raise DkError(rc, "dk_create: " + self.lib.dk_strerror(rc).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.dk_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != DK_OK:
            msg = self.lib.dk_last_error_string(self.h).decode()
            raise DkError(rc, f"{what}: {self.lib.dk_strerror(rc).decode()}: {msg}")

    @staticmethod
    def desc(line_width: int, k: int, variant: int = VARIANT_AUTO,
             residency: int = RESIDENT_HOST, l1_bits: int = 0, bin_target: int = 0) -> InputDesc:
        return InputDesc(line_width, k, CONV_DAKC, variant, residency, l1_bits, bin_target, 0)

    def count_raw(self, ptr: int, nbytes: int, d: InputDesc, on_device: bool = False) -> Table:
        t = Table()
        fn = self.lib.dk_count_device if on_device else self.lib.dk_count
        self._check(fn(self.h, ctypes.c_void_p(ptr), nbytes, ctypes.byref(d), ctypes.byref(t)),
                    "dk_count")
        return t

    def count_format(self, text, fmt: int, k: int, convention: int = 0, line_width: int = 0,
                     variant: int = VARIANT_AUTO, copy: bool = True):
        """Count reads given as FASTQ / FASTA / one per line (dk_count_format);
        returns (CountResult, the line width they were laid out at).  With
        copy=False the host table is released without being copied out and the
        result is (distinct k-mers, k-mer occurrences) instead."""
        ptr, n, keep = _buf_ptr(text)
        d = self.desc(max(line_width, 0), k, variant)
        d.convention = convention
        d.line_width = line_width
        t, w = Table(), ctypes.c_int(0)
        self._check(self.lib.dk_count_format(self.h, ctypes.c_void_p(ptr), n, fmt, ctypes.byref(d),
                                             ctypes.byref(t), ctypes.byref(w)), "dk_count_format")
        try:
            if not copy:
                return (int(t.n), int(t.n_kmers)), int(w.value)
            return self.table_result(t), int(w.value)
        finally:
            self.free_table(t)

    def count_table(self, text, line_width: int, k: int, variant: int = VARIANT_AUTO,
                    residency: int = RESIDENT_HOST) -> Table:
        """dk_count keeping the raw table (release it with free_table)."""
        ptr, n, keep = _buf_ptr(text)
        return self.count_raw(ptr, n, self.desc(line_width, k, variant, residency))

    def histogram(self, t: Table, num_buckets: int):
        """(hist[0..num_buckets), PakMan*'s min bucket) of a table (dk_table_histogram)."""
        hist = np.zeros(num_buckets, np.uint64)
        mb = ctypes.c_uint32(0)
        self._check(self.lib.dk_table_histogram(self.h, ctypes.byref(t), num_buckets,
                                                hist.ctypes.data, ctypes.byref(mb)),
                    "dk_table_histogram")
        return hist, int(mb.value)

    def filter_table(self, t: Table, min_count: int) -> Table:
        """The entries of t with count >= min_count, as a new table (dk_table_filter)."""
        out = Table()
        self._check(self.lib.dk_table_filter(self.h, ctypes.byref(t), min_count, ctypes.byref(out)),
                    "dk_table_filter")
        return out

    def lookup(self, t: Table, queries) -> np.ndarray:
        """Counts of query k-mers in t, 0 when absent (dk_table_lookup)."""
        q = np.ascontiguousarray(queries, dtype=np.uint64)
        out = np.zeros(q.size, np.uint32)
        self._check(self.lib.dk_table_lookup(self.h, ctypes.byref(t), q.ctypes.data, q.size,
                                             out.ctypes.data), "dk_table_lookup")
        return out

    PAIR_DTYPE = np.dtype([("kmer", "<u8"), ("count", "<u4")], align=False)  # 12-byte records

    def pairs(self, t: Table) -> np.ndarray:
        """The table as packed 12-byte (k-mer, count) records (dk_table_pairs)."""
        out = np.zeros(int(t.n), dtype=self.PAIR_DTYPE)
        self._check(self.lib.dk_table_pairs(self.h, ctypes.byref(t), out.ctypes.data),
                    "dk_table_pairs")
        return out

    def free_table(self, t: Table):
        self._check(self.lib.dk_table_free(self.h, ctypes.byref(t)), "dk_table_free")

    def count(self, text, line_width: int, k: int, variant: int = VARIANT_AUTO) -> CountResult:
        """Count the k-mers of `text` (bytes or uint8 array of DAKC lines)."""
        ptr, n, keep = _buf_ptr(text)
        t = self.count_raw(ptr, n, self.desc(line_width, k, variant))
        try:
            nd = int(t.n)
            if nd:
                kmers = np.ctypeslib.as_array(t.kmers, shape=(nd,)).copy()
                counts = np.ctypeslib.as_array(t.counts, shape=(nd,)).copy()
            else:
                kmers, counts = np.zeros(0, np.uint64), np.zeros(0, np.uint32)
            return CountResult(kmers, counts, int(t.n_kmers), int(t.variant_used))
        finally:
            self.free_table(t)
            del keep

    def count_batch_nocopy(self, texts, line_width: int, k: int, variant: int = VARIANT_AUTO,
                           residency: int = RESIDENT_HOST, bin_target: int = 0):
        """dk_count_batch without copying the tables out; returns (n_kmers, n_distinct)."""
        keep = [_buf_ptr(t) for t in texts]
        jobs = (Job * max(1, len(texts)))()
        for j, (ptr, n, _) in enumerate(keep):
            jobs[j].text = ptr
            jobs[j].nbytes = n
        outs = (Table * max(1, len(texts)))()
        d = self.desc(line_width, k, variant, residency, 0, bin_target)
        self._check(self.lib.dk_count_batch(self.h, jobs, len(texts), ctypes.byref(d), outs),
                    "dk_count_batch")
        nk = sum(int(outs[j].n_kmers) for j in range(len(texts)))
        nd = sum(int(outs[j].n) for j in range(len(texts)))
        for j in range(len(texts)):
            if outs[j].handle:
                self.free_table(outs[j])
        return nk, nd

    def count_batch_raw(self, texts, line_width: int, k: int, variant: int = VARIANT_AUTO,
                        residency: int = RESIDENT_HOST):
        """dk_count_batch returning the raw dk_table structs (still owned by the
        engine: copy host tables with table_result, release with free_table)."""
        keep = [_buf_ptr(t) for t in texts]
        jobs = (Job * max(1, len(texts)))()
        for j, (ptr, n, _) in enumerate(keep):
            jobs[j].text = ptr
            jobs[j].nbytes = n
        outs = (Table * max(1, len(texts)))()
        d = self.desc(line_width, k, variant, residency)
        self._check(self.lib.dk_count_batch(self.h, jobs, len(texts), ctypes.byref(d), outs),
                    "dk_count_batch")
        return [outs[j] for j in range(len(texts))]

    @staticmethod
    def table_result(t: Table) -> CountResult:
        """Copy a host-resident dk_table into numpy arrays."""
        nd = int(t.n)
        if nd:
            kmers = np.ctypeslib.as_array(t.kmers, shape=(nd,)).copy()
            counts = np.ctypeslib.as_array(t.counts, shape=(nd,)).copy()
        else:
            kmers, counts = np.zeros(0, np.uint64), np.zeros(0, np.uint32)
        return CountResult(kmers, counts, int(t.n_kmers), int(t.variant_used))

    def count_batch(self, texts, line_width: int, k: int, variant: int = VARIANT_AUTO,
                    l1_bits: int = 0, bin_target: int = 0) -> list[CountResult]:
        """Count each read set of `texts` (one pipeline, memory-bounded waves)."""
        keep = [_buf_ptr(t) for t in texts]
        jobs = (Job * max(1, len(texts)))()
        for j, (ptr, n, _) in enumerate(keep):
            jobs[j].text = ptr
            jobs[j].nbytes = n
        outs = (Table * max(1, len(texts)))()
        d = self.desc(line_width, k, variant, RESIDENT_HOST, l1_bits, bin_target)
        self._check(self.lib.dk_count_batch(self.h, jobs, len(texts), ctypes.byref(d), outs),
                    "dk_count_batch")
        res = []
        try:
            for j in range(len(texts)):
                t = outs[j]
                nd = int(t.n)
                if nd:
                    kmers = np.ctypeslib.as_array(t.kmers, shape=(nd,)).copy()
                    counts = np.ctypeslib.as_array(t.counts, shape=(nd,)).copy()
                else:
                    kmers, counts = np.zeros(0, np.uint64), np.zeros(0, np.uint32)
                res.append(CountResult(kmers, counts, int(t.n_kmers), int(t.variant_used)))
        finally:
            for j in range(len(texts)):
                if outs[j].handle:
                    self.free_table(outs[j])
        return res

    # ------------------------------------------------------------- serving
    def serve_start(self, workers: int = 2, max_batch_jobs: int = 1024):
        self._check(self.lib.dk_serve_start(self.h, workers, max_batch_jobs), "dk_serve_start")
        self._inflight = {}

    def serve_stop(self):
        self._check(self.lib.dk_serve_stop(self.h), "dk_serve_stop")
        self._inflight = {}

    def submit(self, text, line_width: int, k: int, variant: int = VARIANT_AUTO,
               residency: int = RESIDENT_HOST) -> int:
        ptr, n, keep = _buf_ptr(text)
        t = ctypes.c_uint64(0)
        d = self.desc(line_width, k, variant, residency)
        self._check(self.lib.dk_submit(self.h, ctypes.c_void_p(ptr), n, ctypes.byref(d),
                                       ctypes.byref(t)), "dk_submit")
        self._inflight[t.value] = keep  # the text is borrowed until the job completes
        return t.value

    def _take(self, ticket: int, rc: int, t: Table, info: JobInfo):
        if rc == DK_ERR_PENDING or rc == DK_ERR_TIMEOUT:
            return None
        self._inflight.pop(ticket, None)
        self._check(rc, "served job")
        try:
            nd = int(t.n)
            if nd:
                kmers = np.ctypeslib.as_array(t.kmers, shape=(nd,)).copy()
                counts = np.ctypeslib.as_array(t.counts, shape=(nd,)).copy()
            else:
                kmers, counts = np.zeros(0, np.uint64), np.zeros(0, np.uint32)
            res = CountResult(kmers, counts, int(t.n_kmers), int(t.variant_used))
        finally:
            if t.handle:
                self.free_table(t)
        return res, {"queued_us": info.queued_us, "run_us": info.run_us,
                     "batch_jobs": info.batch_jobs, "worker": info.worker}

    def poll(self, ticket: int):
        t, info = Table(), JobInfo()
        return self._take(ticket, self.lib.dk_poll(self.h, ticket, ctypes.byref(t),
                                                   ctypes.byref(info)), t, info)

    def wait(self, ticket: int, timeout_ms: int = 60_000):
        t, info = Table(), JobInfo()
        rc = self.lib.dk_wait(self.h, ticket, timeout_ms, ctypes.byref(t), ctypes.byref(info))
        if rc == DK_ERR_TIMEOUT:
            raise DkError(rc, "dk_wait timed out")
        return self._take(ticket, rc, t, info)

    def wait_raw(self, ticket: int, timeout_ms: int = 60_000):
        """dk_wait returning the raw dk_table (host or device resident; release
        it with free_table) and the job info; None while pending."""
        t, info = Table(), JobInfo()
        rc = self.lib.dk_wait(self.h, ticket, timeout_ms, ctypes.byref(t), ctypes.byref(info))
        if rc == DK_ERR_TIMEOUT:
            raise DkError(rc, "dk_wait timed out")
        if rc == DK_ERR_PENDING:
            return None
        self._inflight.pop(ticket, None)
        self._check(rc, "served job")
        return t, {f: getattr(info, f) for f, _ in info._fields_}

    def wait_nocopy(self, ticket: int, timeout_ms: int = 60_000):
        """Like wait(), but the table is released without being copied out:
        returns (distinct k-mers, k-mer occurrences, job info)."""
        t, info = Table(), JobInfo()
        rc = self.lib.dk_wait(self.h, ticket, timeout_ms, ctypes.byref(t), ctypes.byref(info))
        if rc == DK_ERR_TIMEOUT:
            raise DkError(rc, "dk_wait timed out")
        if rc == DK_ERR_PENDING:
            return None
        self._inflight.pop(ticket, None)
        self._check(rc, "served job")
        n, nk = int(t.n), int(t.n_kmers)
        self.lib.dk_table_free(self.h, ctypes.byref(t))
        return n, nk, {f: getattr(info, f) for f, _ in info._fields_}

    def cancel(self, ticket: int) -> int:
        return int(self.lib.dk_cancel(self.h, ticket))

    def autotune(self, text, line_width: int, k: int) -> dict:
        """Time the count of `text` under a few partition / bin / variant
        choices and keep the fastest for inputs of this shape (dk_autotune);
        later counts with automatic parameters use it."""
        ptr, n, keep = _buf_ptr(text)
        t = Tune()
        d = self.desc(line_width, k, VARIANT_AUTO)
        self._check(self.lib.dk_autotune(self.h, ctypes.c_void_p(ptr), n, ctypes.byref(d),
                                         ctypes.byref(t)), "dk_autotune")
        del keep
        return {f: getattr(t, f) for f, _ in t._fields_}

    def autotune_reset(self) -> None:
        self._check(self.lib.dk_autotune_reset(self.h), "dk_autotune_reset")

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.dk_last_stats(self.h, ctypes.byref(s)), "dk_last_stats")
        return s.as_dict()


def num_lines(text, line_width: int) -> int:
    ptr, n, keep = _buf_ptr(text)
    return int(load_library().dk_num_lines(ctypes.c_void_p(ptr), n, line_width))

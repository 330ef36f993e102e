#!/usr/bin/env python
"""Benchmark: k-mer counting throughput on one GB300 (and N independent replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Workload (default ``large_100m``): seeded synthetic 100 Mbp genome, 20% of it
in 200 repeat families (1-5 kbp, 10-100 copies, 2% divergence), 30x coverage
of 150 bp reads (20,000,000 reads, 3.02 GB of DAKC text), 1% substitutions,
50/50 strand; k = 31.  A "step" counts the whole read set once.

* ``value``  -- k-mers/s with the reads resident in HBM, table left in HBM:
  total k-mer occurrences / the step's device time (CUDA events on the
  engine's stream, first kernel to table complete).  The 3 GB input is far
  larger than L2 (129 MB), so no flush is needed between steps; inputs under
  1 GB (the smaller workloads) get a 512 MB L2 flush before every step.
* ``e2e``    -- the same metric through dk_count with host buffers: pinned
  host reads -> H2D -> count -> D2H of the full table into host memory.
* ``roofline`` -- the dominant kernel's algorithmic bytes / its event time,
  against the measured HBM copy peak; ``pipeline_roofline`` does the same
  for the whole step with B_alg = text + 16 N_k + 12 N_d.
* ``cpu_baseline`` -- DAKC's two phases (owner hash, per-owner sort +
  run-length) on all host threads, on a bounded sample of the same reads.

``--impl reference`` times that CPU implementation alone (rank 0 only).
For N > 1 (torchrun) every rank counts its own copy of the workload: the path
has no exchange step on one GPU, so ranks are independent replicas.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-mers/sec k=31 on 1 GB300, % HBM roofline; p50/p99 job latency batched vs plain"
UNIT = "k-mers/s"
KERNEL_NAMES = ["extract_count", "extract_scatter", "partition_hist", "partition_scatter",
                "bin_count", "compact", "wave_graph", "other"]


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier / max / sum over ranks (gloo over the host; no GPU collective)."""

    def __init__(self, rank, world):
        self.rank, self.world = rank, world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def reduce(self, x: float, op: str) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.06)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(name: str, scale: float):
    from dakc_gb300 import synth
    if name == "large_100m":
        g = int(100_000_000 * scale)
        rs = synth.large_100m(genome_len=g)
        cfg = {"workload": "large_100m", "genome_bp": g, "reads": rs.n_lines, "read_len": 150,
               "k": 31, "coverage": 30, "error_rate": 0.01, "repeat_frac": 0.2,
               "repeat_families": 200}
    elif name == "plain_1m":
        rs = synth.plain_1m()
        cfg = {"workload": "plain_1m", "genome_bp": 1_000_000, "reads": rs.n_lines,
               "read_len": 150, "k": 31, "error_rate": 0.001}
    elif name.startswith("zipf_skew"):
        k = int(name.split("_k")[-1]) if "_k" in name else 31
        rs = synth.zipf_skew(k=k, nreads=int(10_000_000 * scale),
                             background_len=int(50_000_000 * scale), check=scale >= 1.0)
        cfg = {"workload": rs.name, "reads": rs.n_lines, "read_len": 150, "k": k,
               "zipf_s": 1.1, "hot_frac": synth.ZIPF_HOT_FRAC, "templates": synth.ZIPF_TEMPLATES}
    else:
        raise SystemExit(f"unknown workload {name}")
    return rs, cfg


def cpu_sample(rs, cap_reads: int):
    """The reads the CPU counts: all of them (cap_reads <= 0), else the first cap_reads."""
    n = rs.n_lines if cap_reads <= 0 else min(rs.n_lines, cap_reads)
    return rs.text[: n * (rs.line_width + 1)], n


def run_cpu(rs, cap_reads: int, steps: int, warmup: int, threads: int):
    """DAKC's two phases (the oracle port) on `threads` host threads."""
    from oracle import pyoracle
    text, n = cpu_sample(rs, cap_reads)
    times, nk = [], 0
    for i in range(warmup + steps):
        (_, _, nk), secs = pyoracle.dakc_port(text, rs.line_width, rs.k, threads, merge=False)
        if i >= warmup:
            times.append(secs)
    t = float(np.mean(times))
    what = "all" if n == rs.n_lines else f"first {n:,} of"
    return {"value": nk / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} {rs.n_lines:,} reads ({nk:,} k-mers), {threads} PEs as "
                      f"threads, phase 1 + phase 2 as DAKC times them, mean of {steps}",
            "seconds": t, "seconds_all": [round(x, 4) for x in times],
            "same_config": n == rs.n_lines, "reads": n}


def cpu_reads_for(rs, requested: int, runs: int, budget_s: float = 300.0,
                  kmers_per_s: float = 4.0e8) -> int:
    """Reads per CPU step: the whole workload (the same configuration as the
    GPU arm) unless `runs` passes over it would take longer than `budget_s`
    at a conservative `kmers_per_s`; then the largest prefix that fits."""
    if requested > 0:
        return requested
    per_read = max(1, rs.line_width - rs.k + 1)
    fit = int(budget_s * kmers_per_s / max(1, runs) / per_read)
    return 0 if fit >= rs.n_lines else max(1, fit)


def settle_link(max_s: float = 20.0) -> dict:
    """Time 1 GB page-locked copies up and down until three passes in a row
    run within 10% of the best rates seen (at least six passes, at most
    max_s seconds), so that the end-to-end calls start on a quiet host link
    (the host's memory and links are shared; on a box that has just freed
    large page-locked allocations, copies run slow for seconds)."""
    import torch
    n = 1 << 30
    h = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(n, dtype=torch.uint8, device="cuda")
    best_up = best_down = 0.0
    ok = passes = 0
    up = down = 0.0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < max_s:
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        d.copy_(h, non_blocking=True)
        ev[1].record()
        h.copy_(d, non_blocking=True)
        ev[2].record()
        ev[2].synchronize()
        up = n / (ev[0].elapsed_time(ev[1]) / 1e3) / 1e9
        down = n / (ev[1].elapsed_time(ev[2]) / 1e3) / 1e9
        best_up, best_down = max(best_up, up), max(best_down, down)
        passes += 1
        ok = ok + 1 if (up >= 0.9 * best_up and down >= 0.9 * best_down) else 0
        if passes >= 6 and ok >= 3:
            break
    del h, d
    return {"seconds": round(time.perf_counter() - t0, 3), "passes": passes,
            "h2d_gbs": round(up, 1), "d2h_gbs": round(down, 1)}


def job_pool(n: int, seed: int = 4):
    """Read sets with the batched workload's shapes: lognormal read counts
    (median 20,000, sigma 1.5, cap 5M), lengths U[100, 250] padded to 250,
    per-set 0.5-5 Mbp genomes, 0.5% substitutions (the first n of the
    4,096-set sequence)."""
    from concurrent.futures import ThreadPoolExecutor
    from dakc_gb300 import synth
    specs = synth.batch_specs(4096, seed=seed)[:n]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        texts = list(ex.map(lambda s: synth.batch_job_text(s, line_width=250), specs))
    return texts


def pin_texts(texts):
    """Place the read sets in one page-locked host allocation (dk_host_alloc),
    as the engine's ingest expects reads to arrive; returns the buffer (keep
    it alive) and numpy views of each set inside it.  Each set starts on a
    64-byte boundary."""
    import dakc_gb300 as dk
    offs, total = [], 0
    for t in texts:
        offs.append(total)
        total += (t.size + 63) & ~63
    buf = dk.PinnedBuffer(total)
    views = []
    for t, o in zip(texts, offs):
        buf.array[o:o + t.size] = t
        views.append(buf.array[o:o + t.size])
    return buf, views


def pct(xs, p):
    return float(np.percentile(np.asarray(xs, dtype=np.float64), p)) if len(xs) else None


def run_batched(eng, texts, variant, residency=None, call_jobs=0, reps=3, bin_target=0):
    """jobs/s of dk_count_batch over all sets vs one dk_count per set, both
    timed around the C calls with the same table residency (tables are
    released, not copied out).  call_jobs > 0 cuts the batched arm into
    consecutive calls of that many sets, each call's tables released before
    the next (a full 4,096-set batch holds more table than host memory)."""
    import dakc_gb300 as dk
    residency = dk.RESIDENT_HOST if residency is None else residency
    desc = dk.Engine.desc(250, 31, variant, residency, 0, bin_target)
    keep = [dk._buf_ptr(t) for t in texts]
    step = call_jobs if call_jobs > 0 else len(texts)
    calls = [texts[i:i + step] for i in range(0, len(texts), step)]

    def batched():
        nk = nd = 0
        for c in calls:
            a, b = eng.count_batch_nocopy(c, 250, 31, variant, residency, bin_target)
            nk += a
            nd += b
        return nk, nd

    eng.count_batch_nocopy(calls[0], 250, 31, variant, residency, bin_target)  # warm-up
    t_runs, waves, ms_dev, ms_h2d, ms_d2h, launches = [], 0, 0.0, 0.0, 0.0, 0
    packed = fallback = 0
    kms = np.zeros(8)
    for _ in range(reps):
        t0 = time.perf_counter()
        nk = nd = 0
        waves = 0
        ms_dev = ms_h2d = ms_d2h = 0.0
        launches = 0
        packed = fallback = 0
        graph_waves = graph_retries = 0
        kms[:] = 0
        for c in calls:
            a, b = eng.count_batch_nocopy(c, 250, 31, variant, residency, bin_target)
            nk += a
            nd += b
            st = eng.stats()
            waves += st["n_waves"]
            ms_dev += st["ms_device"]
            ms_h2d += st["ms_h2d"]
            ms_d2h += st["ms_d2h"]
            launches += st["kernel_launches"]
            packed += st["n_bins_packed"]
            fallback += st["n_bins_fallback"]
            graph_waves += st["graph_waves"]
            graph_retries += st["graph_retries"]
            kms += np.asarray(st["ms_kernel"])
        t_runs.append(time.perf_counter() - t0)
    t_batch = float(np.median(t_runs))

    def one(ptr, n):
        t = eng.count_raw(ptr, n, desc)
        eng.free_table(t)

    for ptr, n, _ in keep[: min(len(keep), 64)]:
        one(ptr, n)  # warm-up
    lat, p_runs = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        for ptr, n, _ in keep:
            a = time.perf_counter()
            one(ptr, n)
            lat.append(time.perf_counter() - a)
        p_runs.append(time.perf_counter() - t0)
    t_plain = float(np.median(p_runs))
    sub = texts[:16]
    got = eng.count_batch(sub, 250, 31, variant)
    exact = all(np.array_equal(g.kmers, p.kmers) and np.array_equal(g.counts, p.counts)
                for g, p in zip(got, (eng.count(t, 250, 31, variant) for t in sub)))
    return {"jobs": len(texts), "k_mers": nk, "distinct": nd, "exact_vs_plain_subset": bool(exact),
            "residency": "device" if residency == dk.RESIDENT_DEVICE else "host",
            "batched": {"jobs_per_s": len(texts) / t_batch, "kmers_per_s": nk / t_batch,
                        "seconds": t_batch, "seconds_all": [round(x, 5) for x in t_runs],
                        "calls": len(calls), "waves": waves, "ms_device": ms_dev,
                        "ms_h2d": ms_h2d, "ms_d2h": ms_d2h, "kernel_launches": launches,
                        "n_bins_packed": packed, "n_bins_fallback": fallback,
                        "graph_waves": graph_waves, "graph_retries": graph_retries,
                        "kernels_ms": {KERNEL_NAMES[i]: round(float(kms[i]), 3) for i in range(8)}},
            "one_job_per_launch": {"jobs_per_s": len(texts) / t_plain, "kmers_per_s": nk / t_plain,
                                   "seconds": t_plain,
                                   "seconds_all": [round(x, 5) for x in p_runs],
                                   "p50_ms": 1e3 * pct(lat, 50),
                                   "p99_ms": 1e3 * pct(lat, 99)},
            "speedup_jobs_per_s": t_plain / t_batch}


def run_served(texts, rate, n_jobs, variant, workers, max_batch, seed=5, residency=None,
               mem_budget=0, flags=0):
    """Open-loop Poisson arrivals at `rate` jobs/s; sizes drawn from the pool.
    The same arrival stream runs once untimed first, so that every worker's
    device arenas and table pools are at their steady-state sizes.  Tables
    stay where `residency` puts them and are released, not copied out;
    mem_budget (bytes, 0 = 80% of free memory) is the context's admission
    budget, split between the workers."""
    import dakc_gb300 as dk
    from dakc_gb300 import synth
    residency = dk.RESIDENT_HOST if residency is None else residency
    gaps = synth.exponential(seed, n_jobs, rate)
    pick = np.random.Generator(np.random.PCG64(seed)).integers(0, len(texts), n_jobs)

    def stream(eng):
        tickets = []
        t0 = time.perf_counter()
        due = t0
        for i in range(n_jobs):
            due += gaps[i]
            now = time.perf_counter()
            if due > now:
                time.sleep(due - now)
            tickets.append(eng.submit(texts[pick[i]], 250, 31, variant, residency))
        lat, nk, batches = [], 0, []
        for tk in tickets:
            _, n_kmers, info = eng.wait_nocopy(tk, 600_000)  # tables released, not copied
            lat.append((info["queued_us"] + info["run_us"]) / 1e3)
            nk += n_kmers
            batches.append(info["batch_jobs"])
        return time.perf_counter() - t0, lat, nk, batches

    with dk.Engine(0, mem_budget=mem_budget, flags=flags) as eng:
        eng.serve_start(workers=workers, max_batch_jobs=max_batch)
        stream(eng)  # warm-up pass
        span, lat, nk, batches = stream(eng)
        eng.serve_stop()
    return {"rate": rate, "jobs": n_jobs, "jobs_per_s": n_jobs / span, "kmers_per_s": nk / span,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "p999_ms": pct(lat, 99.9),
            "mean_batch_jobs": float(np.mean(batches)), "workers": workers,
            "max_batch": max_batch,
            "residency": "device" if residency == dk.RESIDENT_DEVICE else "host",
            "mem_budget_gb": round(mem_budget / 1e9, 1) if mem_budget else None}


def run_formats(steps: int):
    """The next rows of the path, timed end to end through their C calls on
    the C1-sized read set (100,000 reads of 100-250 bp from a 1 Mbp genome):
    FASTQ -> DAKC lines -> count, FASTA with the PakMan* convention, and the
    table operations (histogram + cut-off, filter, lookups, packed records)
    on the C2 table kept on the device."""
    import dakc_gb300 as dk
    from dakc_gb300 import synth
    spec = synth.batch_specs(1, seed=11)[0]
    spec = synth.JobSpec(spec.job_id, spec.seed, 1_000_000, 100_000)
    text = synth.batch_job_text(spec, line_width=250)
    reads = [bytes(l).rstrip(b"M") for l in text.reshape(-1, 251)[:, :250]]
    fq = b"".join(b"@r%d\n%s\n+\n%s\n" % (i, r, b"I" * len(r)) for i, r in enumerate(reads))
    fa = b"".join(b">r%d\n%s\n" % (i, r) for i, r in enumerate(reads))
    out = {"mode": "formats", "workload": "100,000 reads of 100-250 bp, k = 31"}

    def timed(fn):
        fn()
        t0 = time.perf_counter()
        for _ in range(steps):
            r = fn()
        return (time.perf_counter() - t0) / steps, r

    with dk.Engine(0) as eng:
        for name, buf, fmt, conv in (("fastq_dakc", fq, dk.FORMAT_FASTQ, dk.CONV_DAKC),
                                     ("fasta_pakman", fa, dk.FORMAT_FASTA, dk.CONV_PAKMAN)):
            pin = dk.PinnedBuffer(len(buf))
            pin.array[:] = np.frombuffer(buf, np.uint8)
            # the C call only: the host table it returns is released, not
            # copied into numpy arrays
            sec, ((nd, nk), width) = timed(lambda: eng.count_format(pin.array, fmt, 31, conv,
                                                                    copy=False))
            out[name] = {"input_bytes": len(buf), "line_width": width, "k_mers": nk,
                         "distinct": nd, "ms": 1e3 * sec,
                         "kmers_per_s": nk / sec, "input_gb_per_s": len(buf) / sec / 1e9,
                         "note": "host FASTQ/FASTA in, host table out (dk_count_format; "
                                 "the table is released, not copied to numpy)"}
            pin.free()
        rs, _ = make_workload("large_100m", 1.0)
        t = eng.count_table(rs.text, 150, 31, dk.VARIANT_AUTO, dk.RESIDENT_DEVICE)
        n = int(t.n)
        sec, (hist, mb) = timed(lambda: eng.histogram(t, 256))
        out["histogram_cutoff"] = {"entries": n, "ms": 1e3 * sec, "entries_per_s": n / sec,
                                   "num_buckets": 256, "min_bucket": mb}

        def filt():
            f = eng.filter_table(t, mb)
            kept = int(f.n)
            eng.free_table(f)
            return kept
        sec, kept = timed(filt)
        out["filter"] = {"entries": n, "kept": kept, "ms": 1e3 * sec, "entries_per_s": n / sec}
        q = np.random.Generator(np.random.PCG64(3)).integers(0, 1 << 62, 10_000_000, dtype=np.uint64)
        # page-locked query and result buffers (dk_host_alloc), as a serving
        # caller would hold them
        qpin = dk.PinnedBuffer(q.nbytes)
        opin = dk.PinnedBuffer(q.size * 4)
        qpin.array[:] = q.view(np.uint8)

        def look():
            rc = eng.lib.dk_table_lookup(eng.h, ctypes.byref(t), qpin.ptr, q.size, opin.ptr)
            if rc != dk.DK_OK:
                raise dk.DkError(rc, "dk_table_lookup")
        sec, _ = timed(look)
        qpin.free()
        opin.free()
        out["lookup"] = {"queries": int(q.size), "table": n, "ms": 1e3 * sec,
                         "queries_per_s": q.size / sec,
                         "note": "page-locked host queries in, host counts out"}
        eng.free_table(t)
    return out


def alg_bytes(st: dict, nbytes: int) -> list[float]:
    nk, nd, npart = st["n_kmers"], st["n_distinct"], st["n_partitioned"]
    return [nbytes,                    # extract_count: read the text
            nbytes + 8 * nk,           # extract_scatter: read text, write keys
            8 * npart,                 # partition_hist: read keys
            16 * npart,                # partition_scatter: read + write keys
            8 * nk + 12 * nd,          # bin_count: read keys, write staged pairs
            24 * nd,                   # compact: read + write pairs
            0, 0]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="large_100m")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--variant", default="auto", choices=["auto", "sort", "hash"])
    ap.add_argument("--l1-bits", type=int, default=0, help="level-1 partition bits (0 = auto)")
    ap.add_argument("--bin-target", type=int, default=0, help="keys per bin (0 = auto)")
    ap.add_argument("--cpu-reads", type=int, default=0,
                    help="reads per CPU step (0 = all reads of the workload, the GPU arm's "
                         "configuration, unless that would not finish within about 5 minutes)")
    ap.add_argument("--cpu-steps", type=int, default=3,
                    help="timed runs of the CPU baseline leg in the engine's line")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="count with the automatic parameters instead of the autotuned ones")
    ap.add_argument("--e2e-steps", type=int, default=16)
    ap.add_argument("--mode", default="count", choices=["count", "batch", "serve", "formats"],
                    help="count: the headline line; batch / serve: batched and served forms")
    ap.add_argument("--jobs", type=int, default=256, help="read sets for batch / serve modes")
    ap.add_argument("--rates", default="10,30,100,300,1000,2000")
    ap.add_argument("--serve-jobs", type=int, default=200)
    ap.add_argument("--pageable-jobs", action="store_true",
                    help="batch / serve read sets in pageable memory (staged through pinned slots)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched / served summaries in the headline line")
    ap.add_argument("--residency", default="device", choices=["device", "host"],
                    help="where batch / serve tables stay (both arms alike)")
    ap.add_argument("--call-jobs", type=int, default=0,
                    help="batch mode: sets per dk_count_batch call (0 = all in one call)")
    ap.add_argument("--reps", type=int, default=3, help="batch mode: timed repetitions")
    ap.add_argument("--workers", type=int, default=2, help="serve mode: workers in both arms")
    ap.add_argument("--mem-budget-gb", type=float, default=150.0,
                    help="serve mode: the context's device-memory admission budget")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.mode == "formats" and args.impl == "engine":
        print(json.dumps(run_formats(args.steps)), flush=True)
        return 0

    if args.mode in ("batch", "serve") and args.impl == "engine":
        import dakc_gb300 as dk
        variant = {"auto": dk.VARIANT_AUTO, "sort": dk.VARIANT_SORT,
                   "hash": dk.VARIANT_HASH}[args.variant]
        texts = job_pool(args.jobs)
        pinned = None
        if not args.pageable_jobs:  # reads arrive in page-locked buffers (the engine's ingest)
            pinned, texts = pin_texts(texts)
        res = dk.RESIDENT_DEVICE if args.residency == "device" else dk.RESIDENT_HOST
        if args.mode == "batch":
            with dk.Engine(local) as eng:
                out = run_batched(eng, texts, variant, res, args.call_jobs, args.reps,
                                  args.bin_target)
            out.update(mode="batch", workload="batch_jobs (first %d of 4,096 sets)" % len(texts),
                       reads_in="pageable" if pinned is None else "pinned (dk_host_alloc)")
            print(json.dumps(out), flush=True)
        else:
            budget = int(args.mem_budget_gb * 1e9)
            for r in [float(x) for x in args.rates.split(",")]:
                cb = run_served(texts, r, args.serve_jobs, variant, args.workers, 1024,
                                residency=res, mem_budget=budget)
                one = run_served(texts, r, args.serve_jobs, variant, args.workers, 1,
                                 residency=res, mem_budget=budget)
                print(json.dumps({"mode": "serve", "continuous_batching": cb,
                                  "one_job_per_launch": one}), flush=True)
        return 0

    if args.impl == "reference":
        if rank != 0:
            return 0
        rs, cfg = make_workload(args.workload, args.scale)
        threads = os.cpu_count() or 1
        reads = cpu_reads_for(rs, args.cpu_reads, args.steps + args.warmup)
        cb = run_cpu(rs, reads, args.steps, args.warmup, threads)
        line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": cb["seconds"] * 1000.0, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
                "config": dict(cfg, sample_reads=cb["reads"], same_config=cb["same_config"]),
                "impl": "reference",
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                    "same_config", "seconds_all")},
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    import torch
    import dakc_gb300 as dk

    dist = Dist(rank, world)
    torch.cuda.set_device(local)
    rs, cfg = make_workload(args.workload, args.scale)
    nbytes = rs.text.size
    variant = {"auto": dk.VARIANT_AUTO, "sort": dk.VARIANT_SORT, "hash": dk.VARIANT_HASH}[args.variant]

    eng = dk.Engine(local)
    d_text = torch.empty(nbytes + 64, dtype=torch.uint8, device=f"cuda:{local}")
    d_text[:nbytes].copy_(torch.from_numpy(rs.text))
    torch.cuda.synchronize()
    desc = dk.Engine.desc(rs.line_width, rs.k, variant, dk.RESIDENT_DEVICE, args.l1_bits,
                          args.bin_target)
    # autotuner (before the warm-up, outside the timed region): counts with
    # automatic parameters then use the fastest choice it found for this shape
    tuned = None
    if not args.no_autotune and variant == dk.VARIANT_AUTO and not args.l1_bits \
            and not args.bin_target:
        tuned = eng.autotune(rs.text, rs.line_width, rs.k)

    # inputs that are not far larger than L2 (129 MB): L2 is flushed before
    # every step by writing a 512 MB buffer (outside the engine's timed region)
    flush_buf = None
    if nbytes < (1 << 30):
        flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def step():
        if flush_buf is not None:
            flush_buf.zero_()
            torch.cuda.synchronize()
        t = eng.count_raw(d_text.data_ptr(), nbytes, desc, on_device=True)
        st = eng.stats()
        eng.free_table(t)
        return st

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    sts = [step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    dist.barrier()
    w1 = time.perf_counter()
    clk = clocks.stop()

    dev_ms = float(sum(s["ms_device"] for s in sts))
    nk = sts[0]["n_kmers"]
    nd = sts[0]["n_distinct"]
    t_max = dist.reduce(dev_ms, "max")
    units = dist.reduce(float(nk * args.steps), "sum")
    value = units / (t_max / 1000.0)
    ms_per_step = t_max / args.steps
    launches = int(sum(s["kernel_launches"] for s in sts))

    # kernel roofline from the engine's per-kernel CUDA events
    hbm_peak, peak_kind = peaks()
    kms = np.sum([s["ms_kernel"] for s in sts], axis=0) / args.steps
    kl = np.sum([s["launches_kernel"] for s in sts], axis=0) / args.steps
    ab = alg_bytes(sts[0], nbytes)
    top = int(np.argmax(kms[:7]))
    achieved = ab[top] / (kms[top] / 1000.0) / 1e9 if kms[top] > 0 else 0.0
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        ent = tj.get(KERNEL_NAMES[top])
        if ent and ent.get("bytes_per_kmer"):
            # ncu's DRAM bytes per k-mer of the small case, scaled to this
            # step's k-mers, per launch like alg_bytes_per_launch
            traffic = ent["bytes_per_kmer"] * nk / max(kl[top], 1)
    b_alg = nbytes + 16 * nk + 12 * nd
    pipe = b_alg / (ms_per_step / 1000.0) / 1e9

    # end to end through dk_count: pinned host reads in, host table out
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        pin = dk.PinnedBuffer(nbytes)
        pin.array[:] = rs.text
        hdesc = dk.Engine.desc(rs.line_width, rs.k, variant, dk.RESIDENT_HOST)
        link = settle_link()
        # the first call pins the host table pool; the others settle it
        for _ in range(3):
            eng.free_table(eng.count_raw(pin.ptr, nbytes, hdesc))
        walls, parts = [], []
        for _ in range(args.e2e_steps):
            t0 = time.perf_counter()
            t = eng.count_raw(pin.ptr, nbytes, hdesc)
            walls.append(time.perf_counter() - t0)
            n_out = int(t.n)
            eng.free_table(t)
            st = eng.stats()
            # per call: device time, upload, and the download left after the device
            parts.append([round(st["ms_device"], 2), round(st["ms_h2d"], 2),
                          round(st["ms_d2h"], 2)])
        # the same call with the reads in pageable memory, as the reference's
        # caller holds them (a malloc'd chunk); read in place where the device
        # can, else staged through page-locked slots
        pwalls = []
        for i in range(3 + max(1, args.e2e_steps // 2)):
            t0 = time.perf_counter()
            t = eng.count_raw(rs.text.ctypes.data, nbytes, hdesc)
            if i >= 3:
                pwalls.append(time.perf_counter() - t0)
            eng.free_table(t)
        pst = eng.stats()
        pageable = {"value": nk / float(np.mean(pwalls)), "unit": UNIT,
                    "ms_per_step": float(np.mean(pwalls)) * 1000.0,
                    "ms_median": float(np.median(pwalls)) * 1000.0,
                    "walls_ms": [round(x * 1000.0, 2) for x in pwalls],
                    "read_in_place": bool(pst["upload_in_place"]),
                    "upload_chunks": int(pst["upload_chunks"])}
        w = float(np.mean(walls))
        e2e = {"value": nk / w, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": n_out * 12, "ms_per_step": w * 1000.0,
               "ms_median": float(np.median(walls)) * 1000.0,
               "value_median": nk / float(np.median(walls)),
               "ms_h2d": st["ms_h2d"], "ms_d2h": st["ms_d2h"],
               "walls_ms": [round(x * 1000.0, 2) for x in walls],
               "device_h2d_d2h_ms": parts, "pageable_reads": pageable, "link_settle": link}
        pin.free()

    forms = None
    if rank == 0 and world == 1 and not args.no_forms:
        pinned_forms, texts = pin_texts(job_pool(64))
        budget = int(args.mem_budget_gb * 1e9)
        forms = {"batched": run_batched(eng, texts, variant, dk.RESIDENT_DEVICE),
                 "served": {"continuous_batching": run_served(texts, 2000.0, 64, variant, 2, 1024,
                                                              residency=dk.RESIDENT_DEVICE,
                                                              mem_budget=budget),
                            "one_job_per_launch": run_served(texts, 2000.0, 64, variant, 2, 1,
                                                             residency=dk.RESIDENT_DEVICE,
                                                             mem_budget=budget)},
                 "note": "first 64 sets of the 4,096-set batched workload, tables left on the "
                         "device in both arms; served: Poisson 2,000 jobs/s (the top offered "
                         "rate; --mode serve sweeps 10-2,000), 2 workers in both arms, "
                         f"{args.mem_budget_gb:g} GB admission budget"}

    # CPU baseline last (rank 0, N=1 only), once the GPU is idle: its tens of
    # GB of host buffers are allocated and freed after the end-to-end calls,
    # whose copies share the host's memory (run first, they were followed by
    # slower copies in some of those calls)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = run_cpu(rs, cpu_reads_for(rs, args.cpu_reads, args.cpu_steps), args.cpu_steps, 0,
                      os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded generator; ART-simulated datasets are not available)",
            "config": dict(cfg, variant=args.variant,
                           l2_flush=(f"inputs ({nbytes / 1e9:.2f} GB) larger than L2"
                                     if flush_buf is None else
                                     f"inputs ({nbytes / 1e9:.2f} GB) not larger than L2: "
                                     "512 MB written before every step"),
                           parallelism=f"replicas x{world}",
                           autotuned=({k: tuned[k] for k in ("l1_bits", "bin_target", "variant",
                                                             "candidates")} if tuned else None)),
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[top], "achieved": achieved,
                         "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": traffic,
                         "traffic_over_alg": (traffic / (ab[top] / max(kl[top], 1))
                                              if traffic else None),
                         "peak_kind": peak_kind,
                         "alg_bytes_per_launch": ab[top] / max(kl[top], 1),
                         "ms_per_launch": kms[top] / max(kl[top], 1)},
            "pipeline_roofline": {"b_alg": b_alg, "achieved": pipe, "peak": hbm_peak,
                                  "unit": "GB/s", "frac": pipe / hbm_peak,
                                  "frac_nominal_8tbs": pipe / 8000.0},
            "kernels_ms_per_step": {KERNEL_NAMES[i]: float(kms[i]) for i in range(8)},
            "n_kmers": nk, "n_distinct": nd, "partition_levels": sts[0]["partition_levels"],
            "n_bins": sts[0]["n_bins"], "n_bins_resorted": sts[0]["n_bins_resorted"],
            "n_bins_packed": sts[0]["n_bins_packed"], "n_bins_fallback": sts[0]["n_bins_fallback"],
            "wall_ms_per_step": (w1 - w0) * 1000.0 / args.steps,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": ({k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                  "same_config", "seconds_all")}
                             if cpu else None),
            "forms": forms,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

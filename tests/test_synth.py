"""Seeded workload generator: determinism and shapes (CPU only)."""
import hashlib
import math

import numpy as np

from dakc_gb300 import synth


def test_reads_independent_of_thread_count():
    g = synth.genome_uniform(5, 200_000, threads=1)
    assert np.array_equal(g, synth.genome_uniform(5, 200_000, threads=7))
    a = synth.reads(6, g, 20_000, 100, 150, 150, rc_frac=0.5, err_rate=0.01, threads=1)
    b = synth.reads(6, g, 20_000, 100, 150, 150, rc_frac=0.5, err_rate=0.01, threads=5)
    assert np.array_equal(a, b)


def test_line_format():
    g = synth.genome_uniform(1, 10_000)
    t = synth.reads(2, g, 500, 100, 250, 250, rc_frac=0.5, err_rate=0.0).reshape(500, 251)
    assert (t[:, 250] == ord("\n")).all()
    body = t[:, :250]
    assert set(np.unique(body).tolist()) <= set(b"ACGTM")
    # 'M' only as right padding; lengths within [100, 250]
    lens = (body != ord("M")).sum(axis=1)
    assert lens.min() >= 100 and lens.max() <= 250
    for row, n in zip(body[:50], lens[:50]):
        assert (row[n:] == ord("M")).all()


def test_error_rate_and_strand():
    g = synth.genome_uniform(3, 100_000)
    fwd = synth.reads(4, g, 2000, 150, 150, 150, rc_frac=0.0, err_rate=0.0).reshape(2000, 151)
    gs = bytes(g)
    assert all(bytes(r[:150]) in gs for r in fwd[:100])
    noisy = synth.reads(4, g, 2000, 150, 150, 150, rc_frac=0.0, err_rate=0.01).reshape(2000, 151)
    rate = (noisy[:, :150] != fwd[:, :150]).mean()
    assert 0.008 < rate < 0.012


def test_repeat_genome_fraction():
    g, rep = synth.genome_repeats(9, 5_000_000, nfam=20, lmin=1000, lmax=5000, cmin=10,
                                  cmax=100, repeat_frac=0.2, div=0.02)
    assert g.size == 5_000_000
    assert 0.15 * g.size < rep < 0.3 * g.size
    assert set(np.unique(g).tolist()) <= set(b"ACGT")


def test_lognormal_and_exponential():
    c = synth.lognormal_counts(4, 4096, 20_000, 1.5, 1, 5_000_000)
    assert 15_000 < np.median(c) < 26_000 and c.max() <= 5_000_000 and c.min() >= 1
    e = synth.exponential(5, 100_000, 100.0)
    assert abs(e.mean() - 0.01) < 0.0005


def test_portable_log_exp():
    lib = synth._load()
    for x in (1e-9, 0.1, 0.5, 0.7, 1.0, 2.0, 3.3, 1e6):
        assert math.isclose(lib.dks_log(x), math.log(x), rel_tol=1e-14, abs_tol=1e-15)
    for x in (-20.0, -1.0, -1e-3, 0.0, 0.3, 1.0, 5.5, 40.0):
        assert math.isclose(lib.dks_exp(x), math.exp(x), rel_tol=1e-14)


def test_plain_workload_shape_and_digest():
    rs = synth.plain_1m()
    assert rs.n_lines == 100_000 and rs.text.size == 100_000 * 151
    # the same bytes on every call (and pinned by tests/golden/index.json)
    h = hashlib.sha256(rs.text.tobytes()).hexdigest()
    assert h == hashlib.sha256(synth.plain_1m().text.tobytes()).hexdigest()


def test_zipf_hot_templates():
    bg = synth.genome_uniform(7, 1_000_000)
    t, hot = synth.zipf_reads(8, bg, 200_000, 150, 0.7, 1000, 1.1)
    assert t.size == 200_000 * 151
    assert 0.68 < hot.sum() / 200_000 < 0.72
    assert hot[0] > hot[9] > hot[99]

"""The command-line counter (dakc-gpu), the engine-side caller that stands
where DAKC's driver stands (dakc/src/main/main.cpp:22-54).

Without a GPU: options, usage, the missing-file exit status (2, as DAKC's
reader exits, fqreader.cpp:31-36) and the error when no device is usable.
On the GPU: the table it writes (12-byte records or text) equals the
oracle's, bit for bit, and the figures it prints (global_kmers,
global_distinct_kmers, as DAKC's BENCHMARK build prints them,
kcounter.cpp:500-501) match.
"""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dakc_gb300.h")


@pytest.fixture(scope="module")
def cli():
    from dakc_gb300 import build
    build.build_engine()
    return build.build_cli()


def run(cli, *args, timeout=600):
    return subprocess.run([cli, *map(str, args)], capture_output=True, text=True, timeout=timeout)


def figures(stdout: str) -> dict:
    out = {}
    for key in ("global_kmers", "global_distinct_kmers"):
        m = re.search(rf"^{key}: (\d+)$", stdout, re.M)
        assert m, stdout
        out[key] = int(m.group(1))
    return out


def records(path):
    rec = np.fromfile(path, dtype=np.dtype([("kmer", "<u8"), ("count", "<u4")]))
    return rec["kmer"], rec["count"]


# ---------------------------------------------------------------- no GPU


def test_help(cli):
    r = run(cli, "--help")
    assert r.returncode == 0 and r.stdout.startswith("usage: dakc-gpu -f FILE")


@pytest.mark.parametrize("args", [
    ["-f", HEADER, "-k", "0"],
    ["-f", HEADER, "-k", "33"],
    ["-f", HEADER, "-r", "0"],
    ["-f", HEADER, "--format", "bam"],
    ["-f", HEADER, "--variant", "radix"],
    ["-k", "31"],                                    # no file
    ["-f", HEADER, "extra"],
    ["-f", HEADER, "--keep-on-device", "-o", "x"],  # a device table has no file
])
def test_bad_options(cli, args):
    r = run(cli, *args)
    assert r.returncode == 1 and "usage:" in r.stderr


def test_missing_file_exits_2(cli):
    r = run(cli, "-f", os.path.join(ROOT, "no", "such", "reads.txt"))
    assert r.returncode == 2 and "Could not open the input file" in r.stderr


def test_no_device_is_an_error(cli):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    r = run(cli, "-f", HEADER)
    assert r.returncode == 1 and r.stderr.startswith("dk_create:")


# ---------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["auto", "hash", "sort"])
def test_counts_file_records_equal_oracle(cli, tmp_path, variant):
    from dakc_gb300 import synth
    from oracle import pyoracle
    g = synth.genome_uniform(31, 300_000)
    text = synth.reads(32, g, 40_000, 150, 150, 150, rc_frac=0.5, err_rate=0.01)
    reads = tmp_path / "reads.txt"
    text.tofile(reads)
    out = tmp_path / "table.bin"
    r = run(cli, "-f", reads, "-k", 31, "-r", 150, "--variant", variant, "-o", out)
    assert r.returncode == 0, r.stderr
    assert "kmer counting time:" in r.stdout and "k-mer Length : 31" in r.stdout
    keys, counts, nk = pyoracle.count(text, 150, 31)
    assert figures(r.stdout) == {"global_kmers": nk, "global_distinct_kmers": keys.size}
    got_k, got_c = records(out)
    assert np.array_equal(got_k, keys) and np.array_equal(got_c, counts)


@pytest.mark.gpu
def test_text_table_edges_and_repeat(cli, tmp_path):
    """Breaks, a stop byte, no final newline; k = 5; the text table names the
    bases in DAKC's code (C=0 A=1 T=2 G=3); repeated calls give one table."""
    from oracle import pyoracle
    lines = [b"ACGTNACGTTGCA", b"acgtacgtMACGT", b"GGGGGGGGGGGGG", b"TTTTACGTACGTA"]
    text = b"\n".join(lines)                      # the last terminator is missing
    reads = tmp_path / "reads.txt"
    reads.write_bytes(text)
    tsv = tmp_path / "table.tsv"
    r = run(cli, "-f", reads, "-k", 5, "-r", 13, "--repeat", 3, "--tsv", tsv)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("kmer counting time:") == 3
    keys, counts, nk = pyoracle.count(np.frombuffer(text, np.uint8), 13, 5)
    sym = "CATG"
    want = ["".join(sym[(int(x) >> (2 * (4 - i))) & 3] for i in range(5)) + f"\t{c}"
            for x, c in zip(keys, counts)]
    assert tsv.read_text().splitlines() == want
    assert figures(r.stdout)["global_kmers"] == nk


@pytest.mark.gpu
def test_histogram_and_min_count(cli, tmp_path):
    from dakc_gb300 import synth
    from oracle import pyoracle
    g = synth.genome_uniform(41, 100_000)
    text = synth.reads(42, g, 30_000, 150, 150, 150, rc_frac=0.5, err_rate=0.02)
    reads = tmp_path / "reads.txt"
    text.tofile(reads)
    out = tmp_path / "kept.bin"
    r = run(cli, "-f", reads, "-k", 21, "-r", 150, "--histogram", 64, "--min-count", 3, "-o", out)
    assert r.returncode == 0, r.stderr
    keys, counts, nk = pyoracle.count(text, 150, 21)
    hist, cut = pyoracle.pakman_histogram_cutoff(counts, 64)
    printed = dict(tuple(map(int, ln.split("\t"))) for ln in
                   r.stdout.split("cut-off")[1].splitlines()[1:] if "\t" in ln)
    assert printed == {c: int(hist[c]) for c in range(1, 64) if hist[c]}
    assert int(re.search(r"cut-off (\d+)", r.stdout).group(1)) == cut
    got_k, got_c = records(out)
    keep = counts >= 3
    assert np.array_equal(got_k, keys[keep]) and np.array_equal(got_c, counts[keep])
    assert re.search(rf"kept \(count >= 3\): {int(keep.sum())} distinct, "
                     rf"{int(counts[keep].sum())} k-mers", r.stdout)


@pytest.mark.gpu
def test_fastq_format(cli, tmp_path):
    """FASTQ reads are laid out as fq2txtmaker.sh lays them out, then counted."""
    from oracle import pyoracle
    rng = np.random.Generator(np.random.PCG64(5))
    g = rng.choice(np.frombuffer(b"ACGT", np.uint8), 50_000)
    reads = []
    for i in range(2000):
        L = int(rng.integers(60, 200))
        s = int(rng.integers(0, g.size - L))
        reads.append(g[s:s + L].tobytes())
    fq = b"".join(b"@r%d\n%s\n+\n%s\n" % (i, x, b"I" * len(x)) for i, x in enumerate(reads))
    path = tmp_path / "reads.fq"
    path.write_bytes(fq)
    out = tmp_path / "table.bin"
    r = run(cli, "-f", path, "-k", 25, "--format", "fastq", "-o", out)
    assert r.returncode == 0, r.stderr
    txt, w = pyoracle.fq2txt(fq)
    assert f"Line Width : {w}" in r.stdout
    keys, counts, nk = pyoracle.count(np.frombuffer(txt, np.uint8), w, 25)
    got_k, got_c = records(out)
    assert np.array_equal(got_k, keys) and np.array_equal(got_c, counts)


@pytest.mark.gpu
def test_fasta_pakman_convention(cli, tmp_path):
    """FASTA reads under PakMan*'s convention; the text table names bases in
    PakMan*'s code (A=0 C=1 T=2 G=3)."""
    from oracle import pyoracle
    rng = np.random.Generator(np.random.PCG64(9))
    g = rng.choice(np.frombuffer(b"ACGT", np.uint8), 40_000)
    reads = []
    for i in range(1500):
        L = int(rng.integers(50, 180))
        s = int(rng.integers(0, g.size - L))
        reads.append(g[s:s + L].tobytes())
    fa = b"".join(b">r%d\n%s\n" % (i, x) for i, x in enumerate(reads))
    path = tmp_path / "reads.fa"
    path.write_bytes(fa)
    out, tsv = tmp_path / "table.bin", tmp_path / "table.tsv"
    r = run(cli, "-f", path, "-k", 19, "--format", "fasta", "--pakman", "-o", out, "--tsv", tsv)
    assert r.returncode == 0, r.stderr
    keys, counts, nk = pyoracle.table_of(pyoracle.pakman_kmers(fa, 19))
    got_k, got_c = records(out)
    assert np.array_equal(got_k, keys) and np.array_equal(got_c, counts)
    assert figures(r.stdout)["global_kmers"] == nk
    first = tsv.read_text().splitlines()[0]
    x = int(keys[0])
    assert first == "".join("ACTG"[(x >> (2 * (18 - i))) & 3] for i in range(19)) + f"\t{counts[0]}"


@pytest.mark.gpu
def test_table_kept_on_device(cli, tmp_path):
    """--keep-on-device: the table stays in device memory; the histogram and
    the filter read it there."""
    from dakc_gb300 import synth
    from oracle import pyoracle
    g = synth.genome_uniform(61, 80_000)
    text = synth.reads(62, g, 20_000, 100, 100, 100, rc_frac=0.5, err_rate=0.02)
    reads = tmp_path / "reads.txt"
    text.tofile(reads)
    r = run(cli, "-f", reads, "-k", 27, "-r", 100, "--keep-on-device", "--histogram", 32,
            "--min-count", 2)
    assert r.returncode == 0, r.stderr
    keys, counts, nk = pyoracle.count(text, 100, 27)
    assert figures(r.stdout) == {"global_kmers": nk, "global_distinct_kmers": keys.size}
    hist, cut = pyoracle.pakman_histogram_cutoff(counts, 32)
    printed = dict(tuple(map(int, ln.split("\t"))) for ln in
                   r.stdout.split("cut-off")[1].splitlines()[1:] if "\t" in ln)
    assert printed == {c: int(hist[c]) for c in range(1, 32) if hist[c]}
    keep = counts >= 2
    assert re.search(rf"kept \(count >= 2\): {int(keep.sum())} distinct, "
                     rf"{int(counts[keep].sum())} k-mers", r.stdout)

"""Bit-exact parity at the benchmark configurations' full size.

The headline workloads are counted on the GPU and compared, entry for entry,
with the oracle's table for the same seeded reads:

* large_100m: 100 Mbp genome with repeat families, 20 M reads x 150 bp, k = 31
  (2.4e9 k-mers, 7.9e8 distinct).  Counted from device-resident reads with
  both bin variants (the benchmark's device path), and from page-locked host
  reads into a host table (chunked upload, table streamed out in groups: the
  end-to-end path).
* zipf_skew: 10 M reads x 150 bp, Zipf-skewed hot templates, k in {17, 21, 31}
  (1.2e9-1.34e9 k-mers), both variants.

The oracle is the range-parallel restatement (oracle/dk_oracle.c,
dko_count_mt) on all host cores; it is pinned to the reference's own tables
by tests/test_oracle.py.  Integer work: the bar is exact equality.
"""
import numpy as np
import pytest

import dakc_gb300 as dk
from dakc_gb300 import synth
from oracle import pyoracle

pytestmark = pytest.mark.gpu

VARIANTS = [dk.VARIANT_HASH, dk.VARIANT_SORT]


class _DeviceArray:
    """A device buffer viewed through the CUDA array interface (no copy)."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 3}


def _device_table_to_host(t):
    import torch
    n = int(t.n)
    keys = torch.as_tensor(_DeviceArray(ctypes_addr(t.kmers), n, "<i8"), device="cuda")
    counts = torch.as_tensor(_DeviceArray(ctypes_addr(t.counts), n, "<i4"), device="cuda")
    return keys.cpu().numpy().view(np.uint64), counts.cpu().numpy().view(np.uint32)


def ctypes_addr(p) -> int:
    import ctypes
    return ctypes.cast(p, ctypes.c_void_p).value or 0


def _count_device(engine, text, W, k, variant):
    """dk_count_device: reads resident in HBM, table left in HBM, then copied out."""
    import torch
    d_text = torch.empty(text.size + 64, dtype=torch.uint8, device="cuda")
    d_text[: text.size].copy_(torch.from_numpy(text))
    torch.cuda.synchronize()
    d = dk.Engine.desc(W, k, variant, dk.RESIDENT_DEVICE)
    t = engine.count_raw(d_text.data_ptr(), text.size, d, on_device=True)
    try:
        assert t.on_device == 1
        keys, counts = _device_table_to_host(t)
        return keys, counts, int(t.n_kmers)
    finally:
        engine.free_table(t)
        del d_text


def _assert_same(got, ref):
    keys, counts, nk = got
    rk, rc, rn = ref
    assert nk == rn
    assert keys.size == rk.size, (keys.size, rk.size)
    assert np.array_equal(keys, rk), "k-mer keys differ from the oracle"
    assert np.array_equal(counts, rc), "counts differ from the oracle"


@pytest.fixture(scope="module")
def engine():
    """A context of its own: its arenas (tens of GB at these sizes) are freed
    when the module ends instead of staying with the session's context."""
    with dk.Engine(0) as eng:
        yield eng


@pytest.fixture(scope="module")
def large():
    rs = synth.large_100m()
    ref = pyoracle.count_mt(rs.text, rs.line_width, rs.k)
    assert ref[2] == 20_000_000 * 120
    yield rs, ref


@pytest.mark.parametrize("variant", VARIANTS)
def test_large_100m_device_table(engine, large, variant):
    rs, ref = large
    _assert_same(_count_device(engine, rs.text, rs.line_width, rs.k, variant), ref)
    st = engine.stats()
    assert st["n_kmers"] == ref[2] and st["n_distinct"] == ref[0].size


def test_large_100m_pinned_reads_streamed_host_table(engine, large):
    """The end-to-end path: page-locked reads upload in chunks (each counted
    as it lands) and the host table is copied out group by group."""
    rs, ref = large
    pin = dk.PinnedBuffer(rs.text.size)
    try:
        pin.array[:] = rs.text
        t = engine.count_raw(pin.ptr, rs.text.size, dk.Engine.desc(rs.line_width, rs.k))
        try:
            n = int(t.n)
            assert t.on_device == 0
            keys = np.ctypeslib.as_array(t.kmers, shape=(n,))
            counts = np.ctypeslib.as_array(t.counts, shape=(n,))
            _assert_same((keys, counts, int(t.n_kmers)), ref)
        finally:
            engine.free_table(t)
        st = engine.stats()
        assert st["upload_chunks"] > 1
        assert st["n_groups"] > 1 and st["table_streamed"] == 1
    finally:
        pin.free()


@pytest.fixture(scope="module")
def zipf():
    yield synth.zipf_skew(k=31)


@pytest.mark.parametrize("k", [17, 21, 31])
def test_zipf_skew_full_size(engine, zipf, k):
    text = zipf.text
    ref = pyoracle.count_mt(text, 150, k)
    assert int(ref[1].max()) >= 100_000
    for variant in VARIANTS:
        _assert_same(_count_device(engine, text, 150, k, variant), ref)

"""The C-ABI library: it loads and exports every declared symbol (no GPU needed)."""
import ctypes
import os
import re

import pytest

import dakc_gb300 as dk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dakc_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dk_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for s in ("dk_create", "dk_destroy", "dk_count", "dk_count_device", "dk_table_free",
              "dk_last_stats", "dk_count_small_noalloc"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    lib = dk.load_library()
    for s in declared_symbols():
        assert hasattr(lib, s), f"{s} declared in include/dakc_gb300.h but not exported"
    assert set(declared_symbols()) <= set(dk.ABI_SYMBOLS) | {"dk_count_small_noalloc"}


def test_abi_version_and_strerror():
    lib = dk.load_library()
    lib.dk_abi_version.restype = ctypes.c_int
    assert lib.dk_abi_version() == 1
    assert lib.dk_strerror(dk.DK_ERR_INVALID_ARG) == b"invalid argument"
    assert lib.dk_strerror(dk.DK_ERR_ADMISSION).startswith(b"job exceeds")
    assert lib.dk_strerror(12345) == b"unknown status"


def test_null_context_is_rejected():
    lib = dk.load_library()
    t = dk.Table()
    d = dk.Engine.desc(150, 31)
    assert lib.dk_count(None, None, 0, ctypes.byref(d), ctypes.byref(t)) == dk.DK_ERR_INVALID_ARG
    assert lib.dk_destroy(None) == dk.DK_ERR_INVALID_ARG
    assert lib.dk_table_free(None, ctypes.byref(t)) == dk.DK_ERR_INVALID_ARG


def test_num_lines_host_logic():
    assert dk.num_lines(b"", 5) == 0
    assert dk.num_lines(b"ACGTA\nACGTA\n", 5) == 2
    assert dk.num_lines(b"ACGTA\nACGTA", 5) == 2
    assert dk.num_lines(b"ACGTA\nAC", 5) == dk.DK_ERR_INVALID_ARG
    assert dk.num_lines(b"ACGTA\n\0CGTA\n", 5) == 1
    assert dk.num_lines(b"ACGTA\n", 0) == dk.DK_ERR_INVALID_ARG


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly():
    with pytest.raises(dk.DkError) as e:
        dk.Engine(0)
    assert e.value.status in (dk.DK_ERR_NO_DEVICE, dk.DK_ERR_CUDA)


def test_noalloc_argument_checks_without_gpu():
    lib = dk.load_library()
    f = lib.dk_count_small_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    p = ctypes.c_void_p(16)  # never dereferenced: argument checks run first
    assert f(p, 151, 150, 0, p, p, 200, p, None) == dk.DK_ERR_INVALID_ARG       # bad k
    assert f(p, 100, 150, 31, p, p, 200, p, None) == dk.DK_ERR_INVALID_ARG      # partial line
    assert f(p, 151 * 200, 150, 31, p, p, 10 ** 6, p, None) == dk.DK_ERR_ADMISSION  # > 12,288
    assert f(p, 151 * 10, 150, 31, p, p, 5, p, None) == dk.DK_ERR_INVALID_ARG   # capacity


def test_autotune_rejects_bad_arguments_without_a_device():
    lib = dk.load_library()
    d = dk.Engine.desc(150, 31)
    tune = dk.Tune()
    assert lib.dk_autotune(None, None, 0, ctypes.byref(d), ctypes.byref(tune)) == dk.DK_ERR_INVALID_ARG
    assert lib.dk_autotune_reset(None) == dk.DK_ERR_INVALID_ARG


def _c_struct_fields(name):
    """(field, C type, array length) of `typedef struct {...} name;` in the header."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r"\s*;", src)
    assert m, name
    out = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        parts = decl.split(None, 1)
        ctype, names = parts[0], parts[1]
        for nm in names.split(","):
            nm = nm.strip().lstrip("*")
            a = re.match(r"(\w+)\s*\[(\d+)\]", nm)
            out.append((a.group(1), ctype, int(a.group(2))) if a else (nm, ctype, 1))
    return out


_CTYPES = {"double": ctypes.c_double, "uint64_t": ctypes.c_uint64, "int": ctypes.c_int,
           "uint32_t": ctypes.c_uint32}


@pytest.mark.parametrize("cname,pystruct", [("dk_stats", dk.Stats), ("dk_config", dk.Config),
                                             ("dk_input_desc", dk.InputDesc)])
def test_python_structs_mirror_the_header(cname, pystruct):
    """The ctypes mirrors match the header field by field (order, type, array
    length), so a field added on one side only fails here, not as shifted
    statistics on a GPU machine."""
    cfields = _c_struct_fields(cname)
    pyfields = pystruct._fields_
    assert [f[0] for f in cfields] == [f[0] for f in pyfields]
    for (name, ctype, n), (_, pytype) in zip(cfields, pyfields):
        want = _CTYPES[ctype] * n if n > 1 else _CTYPES[ctype]
        assert ctypes.sizeof(pytype) == ctypes.sizeof(want), name
        if n > 1:
            assert pytype._length_ == n and pytype._type_ == _CTYPES[ctype], name
        else:
            assert pytype == want, name


def test_flags_match_the_header():
    src = open(HEADER).read()
    flags = dict((k, int(v)) for k, v in re.findall(r"#define (DK_FLAG_\w+) (\d+)ull", src))
    assert flags == {"DK_FLAG_STREAM_ALL": dk.FLAG_STREAM_ALL,
                     "DK_FLAG_STAGE_PAGEABLE": dk.FLAG_STAGE_PAGEABLE,
                     "DK_FLAG_NO_GRAPH": dk.FLAG_NO_GRAPH,
                     "DK_FLAG_GRAPH_MIN_BUFFERS": dk.FLAG_GRAPH_MIN_BUFFERS}

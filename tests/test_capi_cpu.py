"""The C-ABI library loads without a GPU, exports every symbol the public
headers declare, and its host-only helpers follow the reference
(src/cl_ops/common/clo_common.c)."""
import ctypes as C
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"typedef[^;]*;", "", text, flags=re.S)
        text = re.sub(r"struct\s+\w+\s*\{.*?\};", "", text, flags=re.S)
        for m in re.finditer(r"\b((?:clo|ccl)_\w+)\s*\(", text):
            if not text[max(0, m.start() - 8):m.start()].strip().endswith("#define"):
                names.add(m.group(1))
        for m in re.finditer(r"extern\s+const\s+[^;(]*?\b((?:clo|ccl)_\w+)\s*(?:\[\s*\])?\s*;", text):
            names.add(m.group(1))
    macros = {"clo_error_quark"}  # also a function
    return sorted(names | macros)


def test_library_exports_every_declared_symbol(clops):
    lib = C.CDLL(str(clops.LIB_PATH))
    names = _declared_functions()
    assert len(names) > 80
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_type_table(clops):
    lib = clops.lib
    names = ["char", "uchar", "short", "ushort", "int", "uint", "long", "ulong",
             "half", "float", "double"]
    sizes = [1, 1, 2, 2, 4, 4, 8, 8, 2, 4, 8]
    for i, (n, s) in enumerate(zip(names, sizes)):
        assert lib.clo_type_get_name(i).decode() == n
        assert lib.clo_type_sizeof(i) == s
        assert clops.call(lib.clo_type_by_name, n.encode()) == i
    with pytest.raises(clops.CloError) as ei:
        clops.call(lib.clo_type_by_name, b"quad")
    assert ei.value.code == clops.CLO_ERROR_UNKNOWN_TYPE


def _ref_nlpo2(x):
    if (x & (x - 1)) & 0xFFFFFFFF == 0:
        return x
    for s in (1, 2, 4, 8, 16):
        x |= x >> s
    return (x + 1) & 0xFFFFFFFF


def test_bit_utilities(clops):
    lib = clops.lib
    for x in [0, 1, 2, 3, 5, 1000, 1 << 20, (1 << 20) + 1, 0x80000000, 0x80000001, 0xFFFFFFFF]:
        assert lib.clo_nlpo2(x) == _ref_nlpo2(x)
        assert lib.clo_ones32(x) == bin(x).count("1")
    for k in range(32):
        assert lib.clo_tzc(1 << k if k < 31 else -(1 << 31)) == k
    assert lib.clo_tzc(0) == 32
    for x in (0, 1, 10, 1000, 100000):
        assert lib.clo_sum(x) == (x * (x + 1) // 2) & 0xFFFFFFFF


def test_error_quark_is_stable(clops):
    assert clops.lib.clo_error_quark() == clops.lib.clo_error_quark() != 0


def test_wrapper_memcheck_starts_clean(clops):
    assert clops.lib.ccl_wrapper_memcheck() == 1

"""Sorters built with custom compare / get_key macros (NVRTC-compiled
kernels): ragged sizes against the oracle's restatement, the program text,
and build errors."""
import numpy as np
import pytest

import oracle
from inputs import keys_of_type
from kats import CUSTOM_FNS

pytestmark = pytest.mark.gpu

CASES = [(0, 5, 5, "((a) < (b))", "(x)"), (2, 5, 5, "((a) > (b))", "((x) & 0xF)"),
         (3, 5, 5, "((a) < (b))", "((x) >> 4)"), (5, 9, 9, "((a) < (b))", "(x)")]


def _run(clops, ctx, q, algo, code, key, cmp, gk, a, out=False):
    s = clops.Sorter(ctx, algo, code, key_type=key, compare=cmp, get_key=gk)
    b = clops.Buffer.from_array(ctx, q, a)
    o = clops.Buffer(ctx, a.nbytes) if out else None
    clops.wait(s.sort_device(q, b, a.size, buf_out=o))
    got = (o or b).read(q, a.dtype, a.size)
    for x in (b, o, s):
        if x is not None:
            x.destroy()
    return got


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"c{c[0]}")
@pytest.mark.parametrize("n", [1, 2, 3, 100, 1000, 4097])
def test_custom_bitonic_and_gselect_ragged(clops, ctx, queue, case, n):
    i, code, key, cmp, gk = case
    key_fn, cmp_fn, _ = CUSTOM_FNS[i]
    a = keys_of_type(40 + n + i, n, {5: np.uint32, 9: np.float32}[code])
    exp = oracle.custom_bitonic(a, key_fn, cmp_fn)
    for algo in ("sbitonic", "abitonic"):
        np.testing.assert_array_equal(_run(clops, ctx, queue, algo, code, key, cmp, gk, a), exp)
    if n <= 1000:
        np.testing.assert_array_equal(
            _run(clops, ctx, queue, "gselect", code, key, cmp, gk, a, out=True),
            oracle.custom_gselect(a, key_fn, cmp_fn))


@pytest.mark.parametrize("n", [5, 4097, 300001])
def test_custom_get_key_satradix_ragged(clops, ctx, queue, n):
    for i, code, key, cmp, gk in CASES[:3]:
        key_fn, _, kdt = CUSTOM_FNS[i]
        a = keys_of_type(50 + n + i, n, np.uint32)
        got = _run(clops, ctx, queue, "satradix", code, key, cmp, gk, a)
        np.testing.assert_array_equal(got, oracle.custom_satradix(a, key_fn, kdt))


def test_key_type_other_than_element_uses_built_kernels(clops, ctx, queue):
    # ulong elements ordered by their low 32 bits (the uint key) with the
    # default compare: bitonic network on the converted keys.
    a = keys_of_type(61, 3000, np.uint64)
    key_fn, cmp_fn, _ = CUSTOM_FNS[4]
    got = _run(clops, ctx, queue, "abitonic", 7, 5, None, None, a)
    np.testing.assert_array_equal(got, oracle.custom_bitonic(a, key_fn, cmp_fn))


def test_custom_program_text_and_build_errors(clops, ctx):
    s = clops.Sorter(ctx, "sbitonic", 5, compare="((a) < (b))")
    src = clops.lib.ccl_program_get_source(clops.lib.clo_sort_get_program(s.h)).decode()
    assert "#define CLO_SORT_COMPARE(a, b) ((a) < (b))" in src
    s.destroy()
    with pytest.raises(clops.CloError) as ei:
        clops.Sorter(ctx, "sbitonic", 5, compare="((a) <<< (b))")
    assert ei.value.code == clops.CLO_ERROR_LIBRARY
    with pytest.raises(clops.CloError) as ei:
        s = clops.Sorter(ctx, "satradix", 5, get_key="((x) & 0xF)")
        try:
            s.sort_kv_host(None, np.zeros(4, np.uint32), np.zeros(4, np.uint32), 5)
        finally:
            s.destroy()
    assert ei.value.code == clops.CLO_ERROR_ARGS

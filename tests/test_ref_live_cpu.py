"""Live comparison of the oracle with the reference's own kernels (run on
host cores through oracle/ref_shim) on inputs beyond the committed known
answers. Needs the reference tree to build oracle/_ref; skipped without."""
import numpy as np
import pytest

import oracle

ref = pytest.importorskip("ref")
if not ref.available():
    pytest.skip("reference tree not available: live comparison skipped",
                allow_module_level=True)

from inputs import keys_of_type  # noqa: E402
from kats import NP  # noqa: E402


@pytest.mark.parametrize("code", [0, 4, 7])
def test_live_satradix_and_bitonic(code):
    a = keys_of_type(901 + code, 1 << 13, NP[code])
    np.testing.assert_array_equal(ref.sort(a, code, "satradix", 128), oracle.radix_sort(a))
    b = keys_of_type(902 + code, 1 << 11, NP[code])
    np.testing.assert_array_equal(ref.sort(b, code, "sbitonic", 64), oracle.bitonic_sort(b, code))


@pytest.mark.parametrize("e,s", [(5, 7), (0, 4), (7, 7)])
def test_live_scan(e, s):
    a = keys_of_type(903 + e, 1 << 17, NP[e])
    np.testing.assert_array_equal(ref.scan(a, e, s, NP[s], 256), oracle.scan(a, e, NP[s]))


@pytest.mark.parametrize("name", ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller",
                                  "tauslcg"])
def test_live_rng(name):
    st = ref.rng_init(name, 3000, 99, 2)
    np.testing.assert_array_equal(st, oracle.rng_init_gid(name, 3000, 99, 1))
    out, st2 = ref.rng_bench(name, st, 3000, 4, 13)
    o_out, o_st = oracle.rng_fill(name, st, 3000, 4, 13)
    np.testing.assert_array_equal(out, o_out)
    np.testing.assert_array_equal(st2, o_st)

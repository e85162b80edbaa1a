"""Object API behaviour on the GPU: registries, option errors with the
reference's error codes, kernel introspection, wrapper bookkeeping, the
bounded-wait watchdog, and full-size property checks."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from inputs import keys_u32, keys_u64, splitmix64

pytestmark = pytest.mark.gpu


def test_unknown_sort_impl(clops, ctx):
    with pytest.raises(clops.CloError) as ei:
        clops.Sorter(ctx, "quicksort", 5)
    assert ei.value.code == clops.CLO_ERROR_IMPL_NOT_FOUND


@pytest.mark.parametrize("algo,opts", [
    ("satradix", "radix=3"), ("satradix", "radix"), ("satradix", "foo=1"),
    ("abitonic", "minps=5"), ("abitonic", "maxps=0"), ("abitonic", "minps=3,maxps=2"),
    ("abitonic", "bar=2")])
def test_bad_options(clops, ctx, algo, opts):
    with pytest.raises(clops.CloError) as ei:
        clops.Sorter(ctx, algo, 5, options=opts)
    assert ei.value.code == clops.CLO_ERROR_ARGS


def test_satradix_bad_scan_impl_fails_at_first_sort(clops, ctx, queue):
    s = clops.Sorter(ctx, "satradix", 5, options="scan=nope")
    b = clops.Buffer.from_array(ctx, queue, keys_u32(1, 100))
    with pytest.raises(clops.CloError) as ei:
        s.sort_device(queue, b, 100)
    assert ei.value.code == clops.CLO_ERROR_IMPL_NOT_FOUND
    b.destroy()
    s.destroy()


def test_custom_snippets_build_and_satradix_ignores_compare(clops, ctx):
    # Custom macros build a program (NVRTC); satradix ignores compare, like
    # the reference, and so needs no program for it.
    s = clops.Sorter(ctx, "abitonic", 5, compare="((a) < (b))")
    assert "CLO_SORT_COMPARE(a, b) ((a) < (b))" in clops.lib.ccl_program_get_source(
        clops.lib.clo_sort_get_program(s.h)).decode()
    s.destroy()
    s = clops.Sorter(ctx, "satradix", 5, compare="((a) < (b))")
    src = clops.lib.ccl_program_get_source(clops.lib.clo_sort_get_program(s.h)).decode()
    assert "clo_jit_keys" not in src
    s.destroy()
    s = clops.Sorter(ctx, "satradix", 5, get_key="((x) >> 1)")
    s.destroy()
    with pytest.raises(clops.CloError) as ei:
        clops.Sorter(ctx, "gselect", 5, get_key="((x) >> )")
    assert ei.value.code == clops.CLO_ERROR_LIBRARY


def test_satradix_rejects_float(clops, ctx):
    with pytest.raises(clops.CloError) as ei:
        clops.Sorter(ctx, "satradix", 9)
    assert ei.value.code == clops.CLO_ERROR_ARGS


def test_kernel_introspection(clops, ctx):
    lib = clops.lib
    for algo, expect in [("sbitonic", 1), ("abitonic", 3), ("gselect", 1), ("satradix", 3)]:
        s = clops.Sorter(ctx, algo, 5)
        nk = clops.call(lib.clo_sort_get_num_kernels, s.h)
        assert nk == expect
        names = [clops.call(lib.clo_sort_get_kernel_name, s.h, i).decode() for i in range(nk)]
        assert all(names)
        for i in range(nk):
            clops.call(lib.clo_sort_get_localmem_usage, s.h, i, 0, 1 << 20)
        assert lib.clo_sort_get_element_size(s.h) == 4
        assert lib.clo_sort_get_key_type(s.h) == 5
        src = lib.ccl_program_get_source(lib.clo_sort_get_program(s.h)).decode()
        assert "CLO_SORT_ELEM_TYPE uint" in src
        s.destroy()
    sc = clops.Scanner(ctx, 5, 7)
    assert lib.clo_scan_get_sum_size(sc.h) == 8
    opts = lib.ccl_program_get_build_options(lib.clo_scan_get_program(sc.h)).decode()
    assert "-DCLO_SCAN_ELEM_TYPE=uint" in opts and "-DCLO_SCAN_SUM_TYPE=ulong" in opts
    sc.destroy()


def test_rng_source_for_client_kernels(clops, ctx, queue):
    rng = clops.Rng(ctx, queue, "mwc64x", clops.CLO_RNG_SEED_DEV_GID, 16)
    src = clops.lib.clo_rng_get_source(rng.h).decode()
    assert src.startswith("#define CLO_RNG_MWC64X") and "clo_rng_next_int" in src
    assert clops.lib.clo_rng_get_size(rng.h) == 16 * 8
    rng.destroy()


def test_profiling_event_duration(clops, ctx, queue):
    a = keys_u32(2, 1 << 20)
    s = clops.Sorter(ctx, "satradix", 5)
    b = clops.Buffer.from_array(ctx, queue, a)
    evt = s.sort_device(queue, b, a.size)
    clops.wait(evt)
    ns = clops.call(clops.lib.ccl_event_get_duration, C.c_void_p(evt))
    assert 0 < ns < 10_000_000_000
    assert clops.lib.ccl_event_get_name(C.c_void_p(evt)) == b"satradix"
    b.destroy()
    s.destroy()


def test_launch_counter_advances(clops, ctx, queue):
    before = clops.launch_count()
    a = keys_u32(3, 50000)
    s = clops.Sorter(ctx, "satradix", 5)
    s.sort_host(queue, a.copy())
    s.destroy()
    assert clops.launch_count() >= before + 5  # upsweep + 4 passes


def test_wrapper_memcheck_after_objects(clops):
    # A private context, queue, buffers and objects; all released.
    ctx = clops.Context(0)
    q = clops.Queue(ctx)
    s = clops.Sorter(ctx, "abitonic", 5)
    b = clops.Buffer.from_array(ctx, q, keys_u32(1, 1000))
    clops.wait(s.sort_device(q, b, 1000))
    rng = clops.Rng(ctx, q, "lcg", clops.CLO_RNG_SEED_DEV_GID, 64)
    rng.destroy()
    b.destroy()
    s.destroy()
    q.destroy()
    ctx.destroy()


def test_lookback_watchdog_reports_and_context_survives(clops, ctx, queue):
    """A tile that never publishes its status: the successors' bounded waits
    run out (about a second), the kernel still ends, the error is reported
    as CLO_ERROR_LIBRARY and the context keeps working. 2^18 elements span
    several tiles whatever the tile size."""
    a = np.ones(1 << 18, dtype=np.uint32)
    sc = clops.Scanner(ctx, 5, 5)
    bi = clops.Buffer.from_array(ctx, queue, a)
    bo = clops.Buffer(ctx, a.nbytes)
    clops.lib.clo_gb300_debug_scan_withhold(0)
    try:
        evt = sc.scan_device(queue, bi, bo, a.size)
        with pytest.raises(clops.CloError) as ei:
            clops.wait(evt)
        assert ei.value.code == clops.CLO_ERROR_LIBRARY
    finally:
        clops.lib.clo_gb300_debug_scan_withhold(-1)
    clops.wait(sc.scan_device(queue, bi, bo, a.size))
    np.testing.assert_array_equal(bo.read(queue, np.uint32, a.size),
                                  np.arange(a.size, dtype=np.uint32))
    for x in (bi, bo, sc):
        x.destroy()


# ----------------------------------------------- full-size checks
@pytest.mark.slow
def test_satradix_5x2pow27_keys_many_tile_waves(clops, ctx, queue):
    """5 x 2^27 + 777 keys: about 47k tiles with a ragged last one, run in
    many waves of CTAs (each waiting only on tiles claimed before it), and
    the upsweep grid sized by its per-thread key cap."""
    n = 5 * (1 << 27) + 777
    a = keys_u32(46, n)
    s = clops.Sorter(ctx, "satradix", 5)
    b = clops.Buffer.from_array(ctx, queue, a)
    clops.wait(s.sort_device(queue, b, n))
    got = b.read(queue, np.uint32, n)
    np.testing.assert_array_equal(
        got, oracle.radix_sort_u32_threaded(a.copy(), os.cpu_count() or 1, 8))
    b.destroy()
    s.destroy()


@pytest.mark.slow
def test_satradix_kv_2pow27_stable_permutation(clops, ctx, queue):
    n = 1 << 27
    k = keys_u64(43, n) & np.uint64(0xFFFF0000000000FF)  # many duplicates
    v = np.arange(n, dtype=np.uint32)
    s = clops.Sorter(ctx, "satradix", 7)
    kb = clops.Buffer.from_array(ctx, queue, k)
    vb = clops.Buffer.from_array(ctx, queue, v)
    clops.wait(s.sort_kv_device(queue, kb, vb, 5, n))
    gk, gv = kb.read(queue, np.uint64, n), vb.read(queue, np.uint32, n)
    assert np.all(gk[1:] >= gk[:-1])
    np.testing.assert_array_equal(k[gv], gk)  # values are the permutation
    same = gk[1:] == gk[:-1]
    assert np.all(gv[1:][same] > gv[:-1][same])  # stable
    for x in (kb, vb, s):
        x.destroy()

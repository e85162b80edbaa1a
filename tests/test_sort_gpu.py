"""GPU parity of the four sorters against the CPU oracle, through the
C-ABI (clo_sort_new / clo_sort_with_device_data / clo_sort_with_host_data),
bit-exact. Sizes cover empty, tiny, ragged (non-multiples of the tile and
of powers of two), one-tile boundaries and multi-tile arrays."""
import numpy as np
import pytest

import oracle
from inputs import keys_of_type, keys_u32, keys_u64, adversarial_u32, low20_u64

pytestmark = pytest.mark.gpu

INT = [(0, np.int8), (1, np.uint8), (2, np.int16), (3, np.uint16), (4, np.int32),
       (5, np.uint32), (6, np.int64), (7, np.uint64)]
ALL = INT + [(8, np.float16), (9, np.float32), (10, np.float64)]


def _sort_dev(clops, ctx, q, algo, code, a, options=None, key_type=None):
    s = clops.Sorter(ctx, algo, code, key_type=key_type, options=options)
    b = clops.Buffer.from_array(ctx, q, a)
    clops.wait(s.sort_device(q, b, a.size))
    out = b.read(q, a.dtype, a.size)
    b.destroy()
    s.destroy()
    return out


# ------------------------------------------------------------- satradix
@pytest.mark.parametrize("code,dt", INT)
@pytest.mark.parametrize("n", [0, 1, 2, 3, 31, 33, 1000, 1023, 1024, 1025, 2559, 2560, 2561,
                               3839, 3840, 3841, 4095, 4096, 4097, 7681, 8191, 8192,
                               8193, 10240, 10241, 14335, 14336, 14337, 15359, 15360, 15361,
                               20481, 28673, 30721,
                               65537, 300001])
def test_satradix_matches_oracle(clops, ctx, queue, code, dt, n):
    a = keys_of_type(100 + n + code, n, dt)
    got = _sort_dev(clops, ctx, queue, "satradix", code, a)
    np.testing.assert_array_equal(got, oracle.radix_sort(a))


# Sorts with at least one large tile per SM take the large tile shape
# (15360 32-bit keys; 10240 64-bit keys; 7168 and 10240 pairs); the sizes
# below put the last tile on each side of a tile boundary.
@pytest.mark.parametrize("code,dt,tile", [(5, np.uint32, 15360), (7, np.uint64, 10240)])
@pytest.mark.parametrize("extra", [-1, 0, 1])
def test_satradix_large_tile_shape_edges(clops, ctx, queue, code, dt, tile, extra):
    n = 160 * tile + extra
    a = keys_of_type(7 + extra + code, n, dt)
    np.testing.assert_array_equal(_sort_dev(clops, ctx, queue, "satradix", code, a),
                                  oracle.radix_sort(a))


@pytest.mark.parametrize("kcode,kdt,vcode,vdt,tile", [
    (7, np.uint64, 5, np.uint32, 7168), (5, np.uint32, 5, np.uint32, 10240),
    (5, np.uint32, 7, np.uint64, 7168), (7, np.uint64, 7, np.uint64, 5120),
    (3, np.uint16, 7, np.uint64, 5120), (1, np.uint8, 5, np.uint32, 10240),
    (2, np.int16, 5, np.uint32, 10240)])
@pytest.mark.parametrize("extra", [-1, 1])
def test_satradix_kv_large_tile_shape_edges(clops, ctx, queue, kcode, kdt, vcode, vdt, tile,
                                            extra):
    n = 160 * tile + extra
    k = keys_of_type(11 + extra, n, kdt)
    v = np.arange(n, dtype=np.uint64).astype(vdt)
    s = clops.Sorter(ctx, "satradix", kcode)
    kb = clops.Buffer.from_array(ctx, queue, k)
    vb = clops.Buffer.from_array(ctx, queue, v)
    clops.wait(s.sort_kv_device(queue, kb, vb, vcode, n))
    rk, rv = oracle.radix_sort(k, v)
    np.testing.assert_array_equal(kb.read(queue, kdt, n), rk)
    np.testing.assert_array_equal(vb.read(queue, vdt, n), rv)
    for b in (kb, vb):
        b.destroy()
    s.destroy()


@pytest.mark.parametrize("code,dt", [(5, np.uint32), (7, np.uint64), (4, np.int32)])
def test_satradix_low_entropy_and_radix_options(clops, ctx, queue, code, dt):
    n = 200003
    a = keys_of_type(5, n, dt)
    a = (a.view(f"u{a.dtype.itemsize}") & np.array(0x00F000F0, dtype=f"u{a.dtype.itemsize}")
         if a.dtype.itemsize >= 4 else a).view(dt)
    ref = oracle.radix_sort(a)
    for opt in (None, "radix=16", "radix=256", "radix=2,scan=blelloch"):
        np.testing.assert_array_equal(_sort_dev(clops, ctx, queue, "satradix", code, a, opt), ref)


def test_satradix_key_type_narrower_than_element(clops, ctx, queue):
    # ulong elements with a uint key: the reference's passes shift the key
    # with OpenCL-masked shifts, so only the low 32 bits order the output.
    n = 70001
    a = keys_u64(9, n)
    got = _sort_dev(clops, ctx, queue, "satradix", 7, a, key_type=5)
    np.testing.assert_array_equal(got, oracle.radix_sort(a, sort_bits=32))


@pytest.mark.parametrize("kind", ["sorted", "reverse", "equal", "distinct16", "zipf"])
def test_satradix_adversarial(clops, ctx, queue, kind):
    a = adversarial_u32(kind, 1 << 20)
    got = _sort_dev(clops, ctx, queue, "satradix", 5, a)
    np.testing.assert_array_equal(got, np.sort(a))


def test_satradix_u64_low20(clops, ctx, queue):
    a = low20_u64(1 << 20)
    np.testing.assert_array_equal(_sort_dev(clops, ctx, queue, "satradix", 7, a), np.sort(a))


@pytest.mark.parametrize("kcode,kdt,vcode,vdt", [
    (5, np.uint32, 5, np.uint32), (7, np.uint64, 5, np.uint32),
    (5, np.uint32, 7, np.uint64), (7, np.uint64, 7, np.uint64), (4, np.int32, 9, np.float32),
    (1, np.uint8, 5, np.uint32), (3, np.uint16, 7, np.uint64)])
@pytest.mark.parametrize("n", [1, 1000, 1023, 1025, 1791, 1792, 1793, 2559, 2561, 4097, 5119,
                               5121, 7167, 7168, 7169, 8193, 10239, 10240, 10241, 14337,
                               20481, 250007])
def test_satradix_kv_stable(clops, ctx, queue, kcode, kdt, vcode, vdt, n):
    k = keys_of_type(31 + n, n, kdt)
    mask = 0x0303 & ((1 << (8 * k.dtype.itemsize)) - 1)
    k = (k.view(f"u{k.dtype.itemsize}") & np.array(mask, dtype=f"u{k.dtype.itemsize}")).view(kdt)
    v = np.arange(n, dtype=np.uint64).astype(vdt)
    s = clops.Sorter(ctx, "satradix", kcode)
    kb = clops.Buffer.from_array(ctx, queue, k)
    vb = clops.Buffer.from_array(ctx, queue, v)
    clops.wait(s.sort_kv_device(queue, kb, vb, vcode, n))
    gk, gv = kb.read(queue, kdt, n), vb.read(queue, vdt, n)
    rk, rv = oracle.radix_sort(k, v)
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv.view(f"u{v.dtype.itemsize}"), rv.view(f"u{v.dtype.itemsize}"))
    for b in (kb, vb):
        b.destroy()
    s.destroy()


def test_satradix_host_data_and_out_buffer(clops, ctx, queue):
    a = keys_u32(77, 123457)
    s = clops.Sorter(ctx, "satradix", 5)
    out = np.empty_like(a)
    s.sort_host(queue, a.copy(), out)
    np.testing.assert_array_equal(out, np.sort(a))
    # data_out != NULL sorts into data_out and leaves data_in untouched.
    bi = clops.Buffer.from_array(ctx, queue, a)
    bo = clops.Buffer(ctx, a.nbytes)
    clops.wait(s.sort_device(queue, bi, a.size, buf_out=bo))
    np.testing.assert_array_equal(bo.read(queue, np.uint32, a.size), np.sort(a))
    np.testing.assert_array_equal(bi.read(queue, np.uint32, a.size), a)
    bi.destroy()
    bo.destroy()
    s.destroy()


# ------------------------------------------------------------- bitonic
@pytest.mark.parametrize("algo", ["sbitonic", "abitonic"])
@pytest.mark.parametrize("code,dt", ALL)
@pytest.mark.parametrize("n", [1, 2, 3, 16, 100, 1024, 16384, 32768, 131075])
def test_bitonic_matches_network_replay(clops, ctx, queue, algo, code, dt, n):
    if algo == "sbitonic" and n > 40000:
        pytest.skip("one launch per step; covered at smaller sizes")
    a = keys_of_type(200 + n + code, n, dt)
    got = _sort_dev(clops, ctx, queue, algo, code, a)
    ref = oracle.bitonic_sort(a, code)
    np.testing.assert_array_equal(got.view(f"u{a.dtype.itemsize}"), ref.view(f"u{a.dtype.itemsize}"))


# Global passes group up to 7 steps (4-byte types), 6 (2-byte) or 5 (1- and
# 8-byte); only stages of 21 steps or more (2^21 elements and up) reach the
# 7-step grouping. 2^21 + 3 elements pad to 2^22.
@pytest.mark.parametrize("code,dt", [(5, np.uint32), (4, np.int32), (9, np.float32),
                                     (3, np.uint16), (0, np.int8), (7, np.uint64)])
def test_abitonic_long_global_passes_match_network_replay(clops, ctx, queue, code, dt):
    n = (1 << 21) + 3
    a = keys_of_type(500 + code, n, dt)
    got = _sort_dev(clops, ctx, queue, "abitonic", code, a)
    ref = oracle.bitonic_sort_threaded(a, code)
    np.testing.assert_array_equal(got.view(f"u{a.dtype.itemsize}"), ref.view(f"u{a.dtype.itemsize}"))


@pytest.mark.parametrize("code,dt", [(8, np.float16), (9, np.float32), (10, np.float64)])
def test_bitonic_non_total_order_is_bit_exact(clops, ctx, queue, code, dt):
    pat = np.array([0.0, -0.0, np.nan, 1.0, -1.0, np.nan, -0.0, 0.0, np.inf, -np.inf], dtype=dt)
    a = np.tile(pat, 6554)[:65536].copy()
    rnd = keys_of_type(3, 65536, dt)
    a[::3] = rnd[::3]
    ref = oracle.bitonic_sort(a, code)
    for algo in ("abitonic",):
        got = _sort_dev(clops, ctx, queue, algo, code, a)
        np.testing.assert_array_equal(got.view(f"u{a.dtype.itemsize}"), ref.view(f"u{a.dtype.itemsize}"))


@pytest.mark.parametrize("opts", ["maxps=1", "maxps=2", "maxps=3,minps=2", "maxsfs=6", "maxsfs=11,maxps=4"])
def test_abitonic_options_do_not_change_result(clops, ctx, queue, opts):
    a = keys_u32(8, 1 << 17)
    got = _sort_dev(clops, ctx, queue, "abitonic", 5, a, options=opts)
    np.testing.assert_array_equal(got, oracle.bitonic_sort(a, 5))


# ------------------------------------------------------------- gselect
@pytest.mark.parametrize("code,dt", ALL)
@pytest.mark.parametrize("n", [1, 2, 7, 1000, 5003])
def test_gselect_matches_oracle(clops, ctx, queue, code, dt, n):
    a = keys_of_type(300 + n, n, dt)
    if np.issubdtype(dt, np.integer):
        a = (a % 13).astype(dt)
    got = _sort_dev(clops, ctx, queue, "gselect", code, a)
    np.testing.assert_array_equal(got, oracle.gselect_sort(a, code))


def test_gselect_kv_stable(clops, ctx, queue):
    n = 4097
    k = (keys_u32(4, n) % 17).astype(np.uint32)
    v = np.arange(n, dtype=np.uint32)
    s = clops.Sorter(ctx, "gselect", 5)
    kb = clops.Buffer.from_array(ctx, queue, k)
    vb = clops.Buffer.from_array(ctx, queue, v)
    clops.wait(s.sort_kv_device(queue, kb, vb, 5, n))
    rk, rv = oracle.gselect_sort(k, 5, v)
    np.testing.assert_array_equal(kb.read(queue, np.uint32, n), rk)
    np.testing.assert_array_equal(vb.read(queue, np.uint32, n), rv)
    kb.destroy()
    vb.destroy()
    s.destroy()


def test_gselect_out_of_place(clops, ctx, queue):
    a = keys_u32(12, 3001)
    s = clops.Sorter(ctx, "gselect", 5)
    bi = clops.Buffer.from_array(ctx, queue, a)
    bo = clops.Buffer(ctx, a.nbytes)
    clops.wait(s.sort_device(queue, bi, a.size, buf_out=bo))
    np.testing.assert_array_equal(bo.read(queue, np.uint32, a.size), np.sort(a))
    np.testing.assert_array_equal(bi.read(queue, np.uint32, a.size), a)
    bi.destroy()
    bo.destroy()
    s.destroy()


# ------------------------------------------ large host-data satradix path
@pytest.mark.parametrize("code,dt,n", [(5, np.uint32, (1 << 22) + 333), (6, np.int64, 1 << 22),
                                       (3, np.uint16, (1 << 23) + 1), (0, np.int8, 1 << 22)])
def test_satradix_host_data_large_matches_oracle(clops, ctx, queue, code, dt, n):
    a = keys_of_type(77 + code, n, dt)
    s = clops.Sorter(ctx, "satradix", code)
    out = np.empty_like(a)
    clops.call(clops.lib.clo_sort_with_host_data, s.h, queue.h, None, clops.np_ptr(a),
               clops.np_ptr(out), n, 0)
    np.testing.assert_array_equal(out, oracle.radix_sort(a))
    s.destroy()


def _pinned(clops, dt, n):
    addr = clops.lib.clo_host_alloc(n * np.dtype(dt).itemsize, None)
    return addr, np.ctypeslib.as_array((clops.C.c_uint8 * (n * np.dtype(dt).itemsize))
                                       .from_address(addr)).view(dt)


# Host-data sorts between page-locked buffers (the bench's end-to-end
# form), across low-entropy inputs that leave most partition groups empty.
@pytest.mark.parametrize("code,dt,n,kind", [
    (5, np.uint32, (1 << 22) + 3, "uniform"), (7, np.uint64, (1 << 23) + 1, "uniform"),
    (5, np.uint32, 1 << 22, "equal"), (5, np.uint32, (1 << 22) + 9, "distinct16"),
    (4, np.int32, (1 << 22) + 5, "uniform")])
def test_satradix_host_data_pinned_output(clops, ctx, queue, code, dt, n, kind):
    if kind == "uniform":
        a = keys_of_type(700 + code, n, dt)
    else:
        a = adversarial_u32(kind, n).view(dt)
    ia, ain = _pinned(clops, dt, n)
    oa, aout = _pinned(clops, dt, n)
    try:
        ain[:] = a
        s = clops.Sorter(ctx, "satradix", code)
        for _ in range(2):
            aout[:] = 0
            clops.call(clops.lib.clo_sort_with_host_data, s.h, queue.h, None, ia, oa, n, 0)
            np.testing.assert_array_equal(aout, oracle.radix_sort(a))
        np.testing.assert_array_equal(ain, a)
        s.destroy()
    finally:
        del ain, aout
        clops.lib.clo_host_free(ia)
        clops.lib.clo_host_free(oa)


def test_satradix_host_data_large_repeated_calls_on_one_sorter(clops, ctx, queue):
    # The pipelined host-data sort keeps its copy stream and events in the
    # sorter: successive calls of different sizes reuse them.
    s = clops.Sorter(ctx, "satradix", 5)
    for i, n in enumerate([(1 << 22) + 3, (1 << 23) + 5, 1 << 22]):
        a = keys_u32(600 + i, n)
        np.testing.assert_array_equal(s.sort_host(queue, a.copy()), np.sort(a))
    s.destroy()


@pytest.mark.parametrize("kind", ["equal", "distinct16", "sorted"])
def test_satradix_host_data_large_low_entropy_and_narrow_key(clops, ctx, queue, kind):
    n = 1 << 22
    a = adversarial_u32(kind, n)
    s = clops.Sorter(ctx, "satradix", 5)
    got = s.sort_host(queue, a.copy())
    np.testing.assert_array_equal(got, oracle.radix_sort(a))
    s.destroy()
    # ulong elements, uint key: stable by the low 32 bits.
    b = (np.arange(n, dtype=np.uint64) << np.uint64(32)) | a.astype(np.uint64)
    s = clops.Sorter(ctx, "satradix", 7, key_type=5)
    got = s.sort_host(queue, b.copy())
    np.testing.assert_array_equal(got, oracle.radix_sort(b, sort_bits=32))
    s.destroy()

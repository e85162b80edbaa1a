"""Segmented sort and scan (clo_sort_segmented_* / clo_scan_segmented_*):
every segment must come out exactly as the oracle's sort / scan of that
segment alone, whatever class (warp, CTA A, CTA B, multi-CTA passes) its
length selects; elements outside the segments stay untouched."""
import numpy as np
import pytest

import oracle
from inputs import keys_of_type, lognormal_lengths, offsets_of, splitmix64

pytestmark = pytest.mark.gpu

UINT, ULONG = 5, 7


def _seg_sort(clops, ctx, q, code, a, off, options=None, key_type=None, buf_extra=0):
    s = clops.Sorter(ctx, "satradix", code, key_type=key_type, options=options)
    b = clops.Buffer.from_array(ctx, q, a)
    ob = clops.Buffer.from_array(ctx, q, np.ascontiguousarray(off, dtype=np.uint64))
    clops.wait(s.sort_segmented_device(q, b, ob, len(off) - 1))
    out = b.read(q, a.dtype, a.size)
    for x in (b, ob, s):
        x.destroy()
    return out


# Lengths that hit every class boundary of every shape (32; class A 512,
# 1024, 2048; class B 2048, 4096, 8192, 16384), the long-segment pass's
# tile edges (10240, 12288, 14336 keys of up to 32 bits; 6144, 7168, 8192
# of 64 bits; one to three tiles), empty and single segments.
EDGE_LENS = [0, 1, 2, 31, 32, 33, 0, 511, 512, 513, 1023, 1024, 1025, 2047, 2048, 2049,
             4095, 4096, 4097, 6143, 6144, 6145, 7167, 7168, 7169, 8191, 8192, 8193,
             10239, 10240, 10241, 12287, 12288, 12289, 14335, 14336, 14337, 16383, 16384,
             16385, 20480, 20481, 24576, 24577, 28672, 28673, 40000, 3, 0, 1]


# Every class A / class B layout, long-pass tile and CTA digit width
# appears in at least one of these shapes (variant = ((a * 3 + b) * 3 + l)
# * 2 + d): the default, 4-bit CTA digits, 256 x 8 class A with a 48-key
# long tile, 256 x 16 class B with a 40-key tile, 1024 x 16 class B with
# 4-bit digits, and the last shape.
SHAPES = [0, 1, ((1 * 3 + 0) * 3 + 1) * 2, ((0 * 3 + 1) * 3 + 2) * 2,
          ((0 * 3 + 2) * 3 + 0) * 2 + 1, 35]


@pytest.mark.parametrize("variant", SHAPES)
@pytest.mark.parametrize("code,dt", [(5, np.uint32), (4, np.int32), (7, np.uint64),
                                     (6, np.int64), (1, np.uint8), (3, np.uint16)])
def test_seg_sort_edge_lengths(clops, ctx, queue, variant, code, dt):
    off = offsets_of(EDGE_LENS, start=5)
    n = int(off[-1]) + 7  # elements before and after the segments
    a = keys_of_type(300 + code, n, dt)
    got = _seg_sort(clops, ctx, queue, code, a, off, options=f"segvariant={variant}")
    np.testing.assert_array_equal(got, oracle.seg_sort(a, off))
    np.testing.assert_array_equal(got[:5], a[:5])
    np.testing.assert_array_equal(got[int(off[-1]):], a[int(off[-1]):])


# Segments of whole long-pass tiles starting at every 16-byte phase of the
# buffer, the last one ending at the buffer's end (no element after it).
@pytest.mark.parametrize("variant,code,dt,tile", [
    (0, 5, np.uint32, 14336), (SHAPES[2], 5, np.uint32, 12288),
    (0, 7, np.uint64, 8192), (SHAPES[3], 7, np.uint64, 6144)])
def test_seg_sort_whole_tiles_at_every_phase_to_the_buffer_end(clops, ctx, queue, variant, code,
                                                                dt, tile):
    # Starts at elements 1, 2 + 2 tiles, 3 + 4 tiles, 4 + 7 tiles (16-byte
    # phases 1, 2, 3, 0 of 32-bit keys; odd, even, odd, even of 64-bit).
    lens = [2 * tile, 1, 2 * tile, 1, 3 * tile, 1, tile, 2 * tile]
    off = offsets_of(lens, start=1)
    n = int(off[-1])
    a = keys_of_type(77 + code, n, dt)
    got = _seg_sort(clops, ctx, queue, code, a, off, options=f"segvariant={variant}")
    np.testing.assert_array_equal(got, oracle.seg_sort(a, off))
    np.testing.assert_array_equal(got[:1], a[:1])


@pytest.mark.parametrize("variant", range(36))
def test_seg_sort_lognormal_u32(clops, ctx, queue, variant):
    lens = lognormal_lengths(3000, 6.0, 2.0, 1, 1 << 18, seed=48)
    off = offsets_of(lens)
    a = keys_of_type(49, int(off[-1]), np.uint32)
    got = _seg_sort(clops, ctx, queue, UINT, a, off, options=f"segvariant={variant}")
    np.testing.assert_array_equal(got, oracle.seg_sort(a, off))


def test_seg_sort_key_narrower_than_element_is_stable(clops, ctx, queue):
    # ulong elements, uint key: segments ordered by the low 32 bits only,
    # equal keys keep their order (the high bits tell them apart).
    lens = [20, 700, 5000, 30000, 1]
    off = offsets_of(lens)
    n = int(off[-1])
    lo = (splitmix64(7, n) >> np.uint64(60))            # 16 distinct low words
    hi = np.arange(n, dtype=np.uint64) << np.uint64(32)  # input order
    a = hi | lo
    got = _seg_sort(clops, ctx, queue, ULONG, a, off, key_type=UINT)
    np.testing.assert_array_equal(got, oracle.seg_sort(a, off, sort_bits=32))


@pytest.mark.parametrize("kind", ["equal", "sorted", "reverse", "distinct16"])
def test_seg_sort_low_entropy(clops, ctx, queue, kind):
    lens = lognormal_lengths(400, 7.0, 1.5, 1, 60000, seed=50)
    off = offsets_of(lens)
    n = int(off[-1])
    a = keys_of_type(51, n, np.uint32)
    if kind == "equal":
        a[:] = 0x9E3779B9
    elif kind == "sorted":
        a = np.sort(a)
    elif kind == "reverse":
        a = np.sort(a)[::-1].copy()
    else:
        a = a & np.uint32(0xF000000F)
    got = _seg_sort(clops, ctx, queue, UINT, a, off)
    np.testing.assert_array_equal(got, oracle.seg_sort(a, off))


def test_seg_sort_host_data_and_no_segments(clops, ctx, queue):
    s = clops.Sorter(ctx, "satradix", UINT)
    lens = [10, 0, 3000, 9000]
    off = offsets_of(lens)
    a = keys_of_type(52, int(off[-1]), np.uint32)
    ref = oracle.seg_sort(a, off)
    got = s.sort_segmented_host(queue, a.copy(), off)
    np.testing.assert_array_equal(got, ref)
    # No segments: nothing happens.
    b = a.copy()
    s.sort_segmented_host(queue, b, np.zeros(1, np.uint64))
    np.testing.assert_array_equal(b, a)
    s.destroy()


def test_seg_sort_rejects_bad_offsets_and_other_sorters(clops, ctx, queue):
    s = clops.Sorter(ctx, "satradix", UINT)
    a = keys_of_type(53, 1000, np.uint32)
    for bad in ([0, 10, 5], [0, 1001], [3, 2]):
        with pytest.raises(clops.CloError) as ei:
            s.sort_segmented_host(queue, a.copy(), np.array(bad, np.uint64))
        assert ei.value.code == clops.CLO_ERROR_ARGS
    # Device form: detected on the device, reported at the next sync.
    b = clops.Buffer.from_array(ctx, queue, a)
    ob = clops.Buffer.from_array(ctx, queue, np.array([0, 10, 5], np.uint64))
    s.sort_segmented_device(queue, b, ob, 2)
    with pytest.raises(clops.CloError) as ei:
        queue.finish()
    assert ei.value.code == clops.CLO_ERROR_ARGS
    for x in (b, ob, s):
        x.destroy()
    g = clops.Sorter(ctx, "gselect", UINT)
    with pytest.raises(clops.CloError) as ei:
        g.sort_segmented_host(queue, a.copy(), np.array([0, 1000], np.uint64))
    assert ei.value.code == clops.CLO_ERROR_ARGS
    g.destroy()
    with pytest.raises(clops.CloError):
        clops.Sorter(ctx, "satradix", UINT, options="segvariant=36")


def test_seg_sort_tune_picks_a_variant_and_keeps_data(clops, ctx, queue):
    s = clops.Sorter(ctx, "satradix", UINT)
    lens = lognormal_lengths(2000, 6.0, 2.0, 1, 1 << 17, seed=54)
    off = offsets_of(lens)
    a = keys_of_type(55, int(off[-1]), np.uint32)
    b = clops.Buffer.from_array(ctx, queue, a)
    ob = clops.Buffer.from_array(ctx, queue, off)
    v, times = s.tune_segmented(queue, b, ob, len(lens))
    assert 0 <= v < clops.SEG_SORT_VARIANTS and s.seg_variant == v
    assert all(t > 0 for t in times) and times[v] == min(times)
    np.testing.assert_array_equal(b.read(queue, np.uint32, a.size), a)
    clops.wait(s.sort_segmented_device(queue, b, ob, len(lens)))
    np.testing.assert_array_equal(b.read(queue, np.uint32, a.size), oracle.seg_sort(a, off))
    for x in (b, ob, s):
        x.destroy()


# ------------------------------------------------------------------ scan
@pytest.mark.parametrize("in_code,in_dt,sum_code,sum_dt", [
    (5, np.uint32, 7, np.uint64), (0, np.int8, 5, np.uint32), (7, np.uint64, 7, np.uint64),
    (4, np.int32, 4, np.int32), (2, np.int16, 6, np.int64), (1, np.uint8, 1, np.uint8)])
def test_seg_scan_edge_lengths(clops, ctx, queue, in_code, in_dt, sum_code, sum_dt):
    off = offsets_of(EDGE_LENS + [100000, 4096 * 3 + 1], start=9)
    n = int(off[-1]) + 13
    a = keys_of_type(400 + in_code, n, in_dt)
    init = keys_of_type(401, n, sum_dt)
    sc = clops.Scanner(ctx, in_code, sum_code)
    bi = clops.Buffer.from_array(ctx, queue, a)
    bo = clops.Buffer.from_array(ctx, queue, init)
    ob = clops.Buffer.from_array(ctx, queue, off)
    clops.wait(sc.scan_segmented_device(queue, bi, bo, ob, len(off) - 1))
    got = bo.read(queue, sum_dt, n)
    np.testing.assert_array_equal(got, oracle.seg_scan(a, off, in_code, sum_dt, out_init=init))
    for x in (bi, bo, ob, sc):
        x.destroy()


def test_seg_scan_lognormal_host_data(clops, ctx, queue):
    lens = lognormal_lengths(5000, 6.0, 2.0, 1, 1 << 18, seed=56)
    off = offsets_of(lens)
    n = int(off[-1])
    a = (splitmix64(57, n) >> np.uint64(56)).astype(np.uint32)
    sc = clops.Scanner(ctx, 5, 7)
    out = np.zeros(n, np.uint64)
    sc.scan_segmented_host(queue, a, out, off)
    np.testing.assert_array_equal(out, oracle.seg_scan(a, off, 5, np.uint64))
    sc.destroy()


# ---------------------------------------------------------------- graphs
def test_segmented_sort_and_scan_replay_from_a_graph(clops, ctx):
    q = clops.Queue(ctx)
    lens = lognormal_lengths(1500, 6.0, 2.0, 1, 1 << 16, seed=58)
    off = offsets_of(lens)
    n = int(off[-1])
    s = clops.Sorter(ctx, "satradix", UINT)
    sc = clops.Scanner(ctx, 5, 7)
    b = clops.Buffer(ctx, n * 4)
    bs = clops.Buffer(ctx, n * 8)
    ob = clops.Buffer.from_array(ctx, q, off)
    # Warm-up outside the capture (first-use setup), then capture.
    b.write(q, keys_of_type(1, n, np.uint32))
    clops.wait(s.sort_segmented_device(q, b, ob, len(lens)))
    g = clops.Graph(q)
    g.begin()
    s.sort_segmented_device(q, b, ob, len(lens))
    sc.scan_segmented_device(q, b, bs, ob, len(lens))
    g.end()
    assert g.num_nodes > 0
    for seed in (60, 61):
        a = keys_of_type(seed, n, np.uint32) >> np.uint32(8)
        b.write(q, a)
        g.launch()
        q.finish()
        srt = oracle.seg_sort(a, off)
        np.testing.assert_array_equal(b.read(q, np.uint32, n), srt)
        np.testing.assert_array_equal(bs.read(q, np.uint64, n),
                                      oracle.seg_scan(srt, off, 5, np.uint64))
    for x in (g, b, bs, ob, s, sc, q):
        x.destroy()


# ------------------------------------------------------ full-size (C4)
@pytest.mark.slow
def test_seg_sort_and_scan_full_size_lognormal(clops, ctx, queue):
    lens = lognormal_lengths(50000, 7.0, 2.0, 1, 1 << 22, seed=48)
    off = offsets_of(lens)
    n = int(off[-1])
    a = keys_of_type(62, n, np.uint32)
    got = _seg_sort(clops, ctx, queue, UINT, a, off)
    np.testing.assert_array_equal(got, oracle.seg_sort(a, off))
    v = (a & np.uint32(0xFF))
    sc = clops.Scanner(ctx, 5, 7)
    out = np.zeros(n, np.uint64)
    sc.scan_segmented_host(queue, v, out, off)
    np.testing.assert_array_equal(out, oracle.seg_scan(v, off, 5, np.uint64))
    sc.destroy()

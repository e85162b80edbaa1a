"""Every configuration the benchmark times, at the size it is timed,
compared element for element with the oracle (or with the reference's own
kernels' digest where they can run it): the radix sort of 2^20 keys with
radix 16, the 2^28 radix sort, the 2^27 key-value sort, the 2^26 bitonic
sort with default options, the adversarial 2^28 / 2^27 distributions, the
2^30 scan and the five generators at 2^24 states x 64 draws.

Inputs are the benchmark's own (same generators, seeds and sizes). The
oracle runs multi-threaded here (the same algorithms as the serial
restatement, identical results: tests/test_oracle_cpu.py), so each check
takes seconds."""
import os

import numpy as np
import pytest

import oracle
from inputs import adversarial_u32, keys_u32, keys_u64, low20_u64, splitmix64
from kats import digest, select

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
THREADS = os.cpu_count() or 1


def _sort(clops, ctx, q, a, algo="satradix", options=None):
    s = clops.Sorter(ctx, algo, {np.uint32: 5, np.uint64: 7}[a.dtype.type], options=options)
    b = clops.Buffer.from_array(ctx, q, a)
    clops.wait(s.sort_device(q, b, a.size))
    got = b.read(q, a.dtype, a.size)
    b.destroy()
    s.destroy()
    return got


def test_radix_2pow20_seed42_radix16_matches_reference_kernels(clops, ctx, queue):
    """2^20 uint32 keys from seed 42, keys only, radix=16: the digest of the
    reference's own satradix kernels on the same input."""
    (k,) = [k for k in select("sort", algo="satradix", code=5, n=1 << 20, seed=42)]
    a = keys_u32(42, 1 << 20)
    got = _sort(clops, ctx, queue, a, options="radix=16")
    assert digest(got) == k["sha256"]
    np.testing.assert_array_equal(got, oracle.radix_sort(a))


def test_radix_2pow28_u32_matches_oracle(clops, ctx, queue):
    a = keys_u32(42, 1 << 28)
    got = _sort(clops, ctx, queue, a)
    np.testing.assert_array_equal(got, oracle.radix_sort_u32_threaded(a.copy(), THREADS, 8))


def test_radix_kv_2pow27_u64_u32_matches_oracle(clops, ctx, queue):
    """(uint64 key from seed 43, uint32 value = original index) pairs. With
    index values the stable order is the stable argsort of the keys."""
    n = 1 << 27
    k = keys_u64(43, n)
    v = np.arange(n, dtype=np.uint32)
    s = clops.Sorter(ctx, "satradix", 7)
    kb = clops.Buffer.from_array(ctx, queue, k)
    vb = clops.Buffer.from_array(ctx, queue, v)
    clops.wait(s.sort_kv_device(queue, kb, vb, 5, n))
    gk, gv = kb.read(queue, np.uint64, n), vb.read(queue, np.uint32, n)
    order = np.argsort(k, kind="stable")
    np.testing.assert_array_equal(gv, order.astype(np.uint32))
    np.testing.assert_array_equal(gk, k[order])
    for x in (kb, vb, s):
        x.destroy()


def test_abitonic_2pow26_default_options_matches_network_replay(clops, ctx, queue):
    """The bitonic configuration as timed: 2^26 uint32 keys from seed 44,
    default options (register-phase tiles, global step groups with strides
    up to 2^25), against the reference network replayed on the host."""
    a = keys_u32(44, 1 << 26)
    got = _sort(clops, ctx, queue, a, algo="abitonic")
    np.testing.assert_array_equal(got, oracle.bitonic_sort_threaded(a, 5, THREADS))


@pytest.mark.parametrize("kind", ["sorted", "reverse", "equal", "distinct16", "zipf"])
def test_radix_adversarial_2pow28_matches_oracle(clops, ctx, queue, kind):
    a = adversarial_u32(kind, 1 << 28)
    got = _sort(clops, ctx, queue, a)
    np.testing.assert_array_equal(got, oracle.radix_sort_u32_threaded(a.copy(), THREADS, 8))


def test_radix_u64_low20_2pow27_matches_sorted(clops, ctx, queue):
    a = low20_u64(1 << 27)
    np.testing.assert_array_equal(_sort(clops, ctx, queue, a), np.sort(a))


def test_scan_2pow30_u32_u64_matches_oracle(clops, ctx, queue):
    n = 1 << 30
    a = np.empty(n, dtype=np.uint32)
    for o in range(0, n, 1 << 24):
        a[o:o + (1 << 24)] = (splitmix64(45, 1 << 24, offset=o) >> np.uint64(56)).astype(np.uint32)
    sc = clops.Scanner(ctx, 5, 7)
    bi = clops.Buffer.from_array(ctx, queue, a)
    bo = clops.Buffer(ctx, n * 8)
    clops.wait(sc.scan_device(queue, bi, bo, n))
    got = bo.read(queue, np.uint64, n)
    for x in (bi, bo, sc):
        x.destroy()
    np.testing.assert_array_equal(got, oracle.scan(a, 5, np.uint64))


@pytest.mark.parametrize("name", ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller"])
def test_rng_2pow24_states_64_draws_matches_oracle(clops, ctx, queue, name):
    """The timed fill: 2^24 host-seeded states (splitmix64 seed 46 bytes;
    Park-Miller states made nonzero), 64 draws. Streams are independent,
    so the oracle replays every 61st state's stream in full and compares
    those columns of the draw-major output, plus the final states."""
    count, draws = 1 << 24, 64
    size = clops.RNG_SEED_SIZE[name]
    seeds = splitmix64(46, count * size // 8 + 1).view(np.uint8)[:count * size].copy()
    if name == "parkmiller":
        w = seeds.view(np.uint32)
        w[:] = (w % 2147483646) + 1
    rng = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_EXT_HOST, count, seeds=seeds)
    out = clops.Buffer(ctx, count * draws * 4)
    clops.wait(rng.fill(queue, out, draws))
    got = out.read(queue, np.uint32, count * draws).reshape(draws, count)
    st = rng.states(queue).reshape(count, size)
    out.destroy()
    rng.destroy()
    pick = np.arange(0, count, 61)
    sub = seeds.reshape(count, size)[pick].reshape(-1)
    ref, ref_st = oracle.rng_fill(name, sub, pick.size, draws)
    np.testing.assert_array_equal(got[:, pick], ref.reshape(draws, pick.size))
    np.testing.assert_array_equal(st[pick].reshape(-1), ref_st)

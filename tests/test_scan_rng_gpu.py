"""GPU parity of the blelloch scanner and the RNGs against the CPU oracle,
through the C-ABI, bit-exact. The RNG cases follow the reference's own
test (src/tests/test_rng.c:48-463): every generator under every seed
type with 10000 seeds, main seed 1234 and hash "(x * 3 + 1)", plus value
checks the reference test does not make."""
import numpy as np
import pytest

import oracle
from inputs import keys_of_type, splitmix64

pytestmark = pytest.mark.gpu

INT = [(0, np.int8), (1, np.uint8), (2, np.int16), (3, np.uint16), (4, np.int32),
       (5, np.uint32), (6, np.int64), (7, np.uint64)]
SUMS = [(1, np.uint8), (3, np.uint16), (5, np.uint32), (7, np.uint64)]


def _scan(clops, ctx, q, a, in_code, out_code, out_dt):
    sc = clops.Scanner(ctx, in_code, out_code)
    bi = clops.Buffer.from_array(ctx, q, a)
    bo = clops.Buffer(ctx, max(a.size, 1) * np.dtype(out_dt).itemsize)
    clops.wait(sc.scan_device(q, bi, bo, a.size))
    out = bo.read(q, out_dt, a.size)
    bi.destroy()
    bo.destroy()
    sc.destroy()
    return out


@pytest.mark.parametrize("code,dt", INT)
@pytest.mark.parametrize("ocode,odt", SUMS)
def test_scan_types(clops, ctx, queue, code, dt, ocode, odt):
    n = 20011
    a = keys_of_type(40 + code, n, dt)
    np.testing.assert_array_equal(_scan(clops, ctx, queue, a, code, ocode, odt),
                                  oracle.scan(a, code, odt))


@pytest.mark.parametrize("n", [0, 1, 2, 511, 512, 513, 4095, 4096, 4097, 8191, 8192, 8193,
                               16385, 131072, 1000003, 5000011])
def test_scan_sizes_uint_to_ulong(clops, ctx, queue, n):
    a = (splitmix64(45, n) >> np.uint64(56)).astype(np.uint32)  # values in [0, 255]
    np.testing.assert_array_equal(_scan(clops, ctx, queue, a, 5, 7, np.uint64),
                                  oracle.scan(a, 5, np.uint64))


@pytest.mark.parametrize("code,dt,ocode,odt", [(1, np.uint8, 1, np.uint8), (0, np.int8, 4, np.int32),
                                               (3, np.uint16, 7, np.uint64), (4, np.int32, 4, np.int32),
                                               (7, np.uint64, 7, np.uint64), (6, np.int64, 2, np.int16)])
def test_scan_many_tiles_per_cta(clops, ctx, queue, code, dt, ocode, odt):
    # More tiles than resident CTAs: CTAs take second and later tiles, whose
    # loads are prefetched and aggregates published during the lookback.
    n = (1 << 22) + 3
    a = keys_of_type(77 + code, n, dt)
    np.testing.assert_array_equal(_scan(clops, ctx, queue, a, code, ocode, odt),
                                  oracle.scan(a, code, odt))


def test_scan_host_data_and_unaligned_views(clops, ctx, queue):
    a = (splitmix64(1, 99999) >> np.uint64(40)).astype(np.uint32)
    sc = clops.Scanner(ctx, 5, 7)
    out = np.empty(a.size, dtype=np.uint64)
    sc.scan_host(queue, a, out)
    np.testing.assert_array_equal(out, oracle.scan(a, 5, np.uint64))
    sc.destroy()


def test_scan_rejects_options_like_reference(clops, ctx):
    with pytest.raises(clops.CloError) as ei:
        clops.Scanner(ctx, 5, 5, options="foo=1")
    assert ei.value.code == clops.CLO_ERROR_ARGS
    with pytest.raises(clops.CloError) as ei:
        clops.Scanner(ctx, 5, 5, algo="hillis")
    assert ei.value.code == clops.CLO_ERROR_IMPL_NOT_FOUND


# ------------------------------------------------------------------ RNG
NUM_SEEDS, INIT_SEED, TEST_HASH = 10000, 1234, "(x * 3 + 1)"


def _hash_ref(kind, x):
    """Python evaluation of the hash texts used below."""
    M = 0xFFFFFFFFFFFFFFFF
    if kind in (None, "", "x", TEST_HASH):
        return x
    if kind == "KNUTH(x)":
        return (x * 2654435761) % 0x100000000
    if kind == "XS1(x)":
        for _ in range(2):
            x = (((x >> 16) ^ x) * 0x45d9f3b) & M
        return (x >> 16) ^ x
    if kind == "x = x << 2":
        return (x << 2) & M
    if kind == "x ^= 0xABCDEF; x = x * 3 + (x >> 7) % 11":
        x ^= 0xABCDEF
        return (x * 3 + (x >> 7) % 11) & M
    raise ValueError(kind)


def _state_from_seed(name, s):
    M = 0xFFFFFFFF
    if name in ("lcg", "xorshift64"):
        return np.array([s], dtype=np.uint64).view(np.uint8)
    if name == "xorshift128":
        return np.array([s & M, (s >> 16) & M, (s >> 32) & M, (s >> 46) & M], dtype=np.uint32).view(np.uint8)
    if name == "mwc64x":
        return np.array([s], dtype=np.uint64).view(np.uint8)
    if name == "parkmiller":
        return np.array([s & M], dtype=np.uint32).view(np.uint8)
    if name == "tauslcg":
        return np.array([s, s], dtype=np.uint64).view(np.uint8)


@pytest.mark.parametrize("name", oracle.GEN.keys())
def test_rng_dev_gid_like_reference_test(clops, ctx, queue, name):
    rng = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_DEV_GID, NUM_SEEDS, INIT_SEED, TEST_HASH)
    st = rng.states(queue)
    np.testing.assert_array_equal(st, oracle.rng_init_gid(name, NUM_SEEDS, INIT_SEED, 0))
    out = clops.Buffer(ctx, NUM_SEEDS * 4 * 3)
    clops.wait(rng.fill(queue, out, 3))
    ref, ref_st = oracle.rng_fill(name, st, NUM_SEEDS, 3)
    np.testing.assert_array_equal(out.read(queue, np.uint32, 3 * NUM_SEEDS), ref)
    np.testing.assert_array_equal(rng.states(queue), ref_st)
    out.destroy()
    rng.destroy()


@pytest.mark.parametrize("name", oracle.GEN.keys())
@pytest.mark.parametrize("hash", [None, "KNUTH(x)", "XS1(x)", "x = x << 2",
                                  "x ^= 0xABCDEF; x = x * 3 + (x >> 7) % 11"])
def test_rng_hashes(clops, ctx, queue, name, hash):
    n = 777
    rng = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_DEV_GID, n, 99, hash)
    st = rng.states(queue)
    exp = np.concatenate([_state_from_seed(name, _hash_ref(hash, i + 99)) for i in range(n)])
    np.testing.assert_array_equal(st, exp)
    rng.destroy()


def test_rng_bad_hash_is_rejected(clops, ctx, queue):
    with pytest.raises(clops.CloError) as ei:
        clops.Rng(ctx, queue, "lcg", clops.CLO_RNG_SEED_DEV_GID, 10, 0, "y = x")
    assert ei.value.code == clops.CLO_ERROR_ARGS


@pytest.mark.parametrize("name", oracle.GEN.keys())
def test_rng_host_mt(clops, ctx, queue, name):
    rng = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_HOST_MT, NUM_SEEDS, INIT_SEED)
    size = NUM_SEEDS * oracle.SEED_SIZE[name]
    np.testing.assert_array_equal(rng.states(queue), oracle.mt19937(INIT_SEED, size // 4).view(np.uint8))
    rng.destroy()


@pytest.mark.parametrize("name", oracle.GEN.keys())
def test_rng_ext_host_and_ext_dev(clops, ctx, queue, name):
    size = NUM_SEEDS * oracle.SEED_SIZE[name]
    # test_rng.c:373-374 seed bytes: ((i + 1) * 3) & 0xFF
    seeds = (((np.arange(size) + 1) * 3) & 0xFF).astype(np.uint8)
    rng = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_EXT_HOST, NUM_SEEDS, seeds=seeds)
    np.testing.assert_array_equal(rng.states(queue), seeds)
    out = clops.Buffer(ctx, NUM_SEEDS * 4 * 4)
    clops.wait(rng.fill(queue, out, 4, bits=17))
    ref, _ = oracle.rng_fill(name, seeds, NUM_SEEDS, 4, 17)
    np.testing.assert_array_equal(out.read(queue, np.uint32, 4 * NUM_SEEDS), ref)
    rng.destroy()
    dev = clops.Buffer.from_array(ctx, queue, seeds)
    rng2 = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_EXT_DEV, NUM_SEEDS, seeds=dev)
    clops.wait(rng2.fill(queue, out, 4, maxint=1000))
    ref2, _ = oracle.rng_fill(name, seeds, NUM_SEEDS, 4, 32, 1000)
    np.testing.assert_array_equal(out.read(queue, np.uint32, 4 * NUM_SEEDS), ref2)
    rng2.destroy()
    dev.destroy()  # the RNG object took its own reference
    out.destroy()


def test_rng_ext_dev_too_small(clops, ctx, queue):
    small = clops.Buffer(ctx, 16)
    with pytest.raises(clops.CloError) as ei:
        clops.Rng(ctx, queue, "xorshift128", clops.CLO_RNG_SEED_EXT_DEV, 100, seeds=small)
    assert ei.value.code == clops.CLO_ERROR_ARGS
    small.destroy()


def test_rng_streams_continue_across_fills(clops, ctx, queue):
    n = 4096 * 3 + 1
    seeds = splitmix64(46, n).view(np.uint8)
    rng = clops.Rng(ctx, queue, "xorshift64", clops.CLO_RNG_SEED_EXT_HOST, n, seeds=seeds)
    out = clops.Buffer(ctx, n * 4 * 8)
    clops.wait(rng.fill(queue, out, 3))
    a = out.read(queue, np.uint32, 3 * n)
    clops.wait(rng.fill(queue, out, 5))
    b = out.read(queue, np.uint32, 5 * n)
    ref, _ = oracle.rng_fill("xorshift64", seeds, n, 8)
    np.testing.assert_array_equal(np.concatenate([a, b]), ref)
    out.destroy()
    rng.destroy()


def test_rng_unknown_and_bad_seed_args(clops, ctx, queue):
    with pytest.raises(clops.CloError) as ei:
        clops.Rng(ctx, queue, "philox", clops.CLO_RNG_SEED_DEV_GID, 10)
    assert ei.value.code == clops.CLO_ERROR_IMPL_NOT_FOUND
    with pytest.raises(clops.CloError) as ei:
        clops.Rng(ctx, queue, "lcg", clops.CLO_RNG_SEED_EXT_HOST, 10, seeds=None)
    assert ei.value.code == clops.CLO_ERROR_ARGS


# ------------------------------------------ large host-data scans (chunked)
@pytest.mark.parametrize("in_code,in_dt,sum_code,sum_dt,n", [
    (5, np.uint32, 7, np.uint64, (1 << 22) + 12345),
    (0, np.int8, 4, np.int32, (1 << 25) + 7),
    (7, np.uint64, 7, np.uint64, 1 << 24),
    (4, np.int32, 5, np.uint32, (1 << 24) + (1 << 23))])
def test_scan_host_data_large_matches_oracle(clops, ctx, queue, in_code, in_dt, sum_code,
                                             sum_dt, n):
    a = keys_of_type(900 + in_code, n, in_dt)
    out = np.zeros(n, sum_dt)
    sc = clops.Scanner(ctx, in_code, sum_code)
    sc.scan_host(queue, a, out)
    np.testing.assert_array_equal(out, oracle.scan(a, in_code, sum_dt))
    sc.destroy()


def test_scan_host_data_large_repeated_calls_on_one_scanner(clops, ctx, queue):
    # The chunked host-data scan keeps its copy streams and events in the
    # scanner: a larger call after a smaller one needs more events.
    sc = clops.Scanner(ctx, 5, 7)
    for i, n in enumerate([(1 << 22) + 1, (1 << 25) + 99, (1 << 23) + 17]):
        a = keys_of_type(950 + i, n, np.uint32)
        out = np.zeros(n, np.uint64)
        sc.scan_host(queue, a, out)
        np.testing.assert_array_equal(out, oracle.scan(a, 5, np.uint64))
    sc.destroy()

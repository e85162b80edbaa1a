"""The CPU oracle, checked against independent implementations (numpy) and
published known-answer values. No GPU needed."""
import numpy as np
import pytest

import oracle
from inputs import splitmix64, keys_u32, keys_of_type

INT_TYPES = [(0, np.int8), (1, np.uint8), (2, np.int16), (3, np.uint16),
             (4, np.int32), (5, np.uint32), (6, np.int64), (7, np.uint64)]


def test_splitmix64_matches_c_and_published_value():
    # splitmix64 with state 0: first output 0xE220A8397B1DCDAF (Vigna's
    # reference implementation).
    assert int(oracle.splitmix64(0, 1)[0]) == 0xE220A8397B1DCDAF
    np.testing.assert_array_equal(oracle.splitmix64(42, 1000), splitmix64(42, 1000))


def test_mt19937_known_answers():
    # init_genrand(5489) known answers (Matsumoto & Nishimura mt19937ar).
    assert list(oracle.mt19937(5489, 3)) == [3499211612, 581869302, 3890346734]
    # 10000th output for the default seed is 4123659995 (C++11 std::mt19937).
    assert int(oracle.mt19937(5489, 10000)[-1]) == 4123659995
    for seed in (0, 1, 1234, 0xFFFFFFFF):
        ref = np.random.RandomState(seed)._bit_generator.random_raw(2000).astype(np.uint32)
        np.testing.assert_array_equal(oracle.mt19937(seed, 2000), ref)


@pytest.mark.parametrize("code,dt", INT_TYPES)
@pytest.mark.parametrize("n", [0, 1, 2, 3, 31, 33, 1000, 4099])
def test_radix_oracle_is_stable_unsigned_sort(code, dt, n):
    k = keys_of_type(7 + n, n, dt)
    # Low-entropy keys too, so that stability matters.
    k = (k.view(f"u{k.dtype.itemsize}") & np.array(0x0F0F, dtype=f"u{k.dtype.itemsize}")).view(dt) \
        if k.dtype.itemsize >= 2 else k
    v = np.arange(n, dtype=np.uint32)
    sk, sv = oracle.radix_sort(k, v)
    u = k.view(f"u{k.dtype.itemsize}")
    order = np.argsort(u, kind="stable")
    np.testing.assert_array_equal(sk, k[order])
    np.testing.assert_array_equal(sv, v[order])


def test_radix_oracle_sort_bits_subset():
    k = keys_of_type(3, 5000, np.uint64)
    v = np.arange(5000, dtype=np.uint32)
    sk, sv = oracle.radix_sort(k, v, sort_bits=32)
    order = np.argsort(k & np.uint64(0xFFFFFFFF), kind="stable")
    np.testing.assert_array_equal(sk, k[order])
    np.testing.assert_array_equal(sv, v[order])


def test_threaded_radix_equals_serial():
    k = keys_u32(42, 1 << 16)
    for bits in (4, 8):
        np.testing.assert_array_equal(oracle.radix_sort_u32_threaded(k.copy(), 4, bits), np.sort(k))


def _py_bitonic(a, gt):
    """Literal replay of the sbitonic host loop + kernel in Python."""
    a = list(a)
    N = len(a)
    stages = N.bit_length() - 1
    for stage in range(1, stages + 1):
        for step in range(stage, 0, -1):
            stride = 1 << (step - 1)
            for gid in range(N // 2):
                i1 = gid + (gid // stride) * stride
                i2 = i1 + stride
                desc = (gid >> (stage - 1)) & 1
                if bool(gt(a[i1], a[i2])) ^ bool(desc):
                    a[i1], a[i2] = a[i2], a[i1]
    return a


@pytest.mark.parametrize("code,dt", INT_TYPES + [(9, np.float32), (10, np.float64), (8, np.float16)])
def test_bitonic_oracle_sorts_and_replays_network(code, dt):
    for n in (1, 2, 16, 64, 100, 1024):
        a = keys_of_type(11 + n, n, dt)
        got = oracle.bitonic_sort(a, code)
        np.testing.assert_array_equal(np.sort(a), got)
    # Exact network replay on values where the compare is not total.
    if np.issubdtype(dt, np.floating):
        a = np.array([0.0, -0.0, np.nan, 1.0, -1.0, np.nan, -0.0, 0.0] * 4, dtype=dt)
        got = oracle.bitonic_sort(a, code)
        ref = np.array(_py_bitonic(a, lambda x, y: x > y), dtype=dt)
        np.testing.assert_array_equal(got.view(f"u{a.dtype.itemsize}"),
                                      ref.view(f"u{a.dtype.itemsize}"))


@pytest.mark.parametrize("code,dt", INT_TYPES + [(9, np.float32), (10, np.float64), (8, np.float16)])
def test_threaded_bitonic_equals_serial_replay(code, dt):
    """The threaded replay (gid-range steps, block-local short strides)
    gives the serial replay's bytes, NaN and signed-zero orders included,
    on sizes below, at and above the block and ragged ones (padding)."""
    for n in (1, 3, 1000, (1 << 14) + 3, 1 << 16, 100003):
        a = keys_of_type(77 + n, n, dt)
        if np.issubdtype(dt, np.floating):
            a[::97] = np.nan
            a[::101] = -0.0
        for threads in (1, 3, 8):
            got = oracle.bitonic_sort_threaded(a, code, threads)
            assert got.tobytes() == oracle.bitonic_sort(a, code).tobytes(), (n, threads)


@pytest.mark.parametrize("code,dt", INT_TYPES + [(9, np.float32)])
def test_gselect_oracle_is_stable_sort(code, dt):
    for n in (1, 5, 300):
        a = keys_of_type(5 + n, n, dt)
        if np.issubdtype(dt, np.integer):
            a = (a % 7).astype(dt)
        v = np.arange(n, dtype=np.uint32)
        out, vout = oracle.gselect_sort(a, code, v)
        order = np.argsort(a, kind="stable")
        np.testing.assert_array_equal(out, a[order])
        np.testing.assert_array_equal(vout, v[order])


@pytest.mark.parametrize("code,dt", INT_TYPES)
@pytest.mark.parametrize("out_dt", [np.uint8, np.uint16, np.uint32, np.uint64])
def test_scan_oracle_matches_numpy(code, dt, out_dt):
    n = 3000
    a = keys_of_type(9, n, dt)
    got = oracle.scan(a, code, out_dt)
    # C conversion of the element to the sum type, then modular sums.
    conv = a.astype(np.int64).astype(np.uint64) if np.issubdtype(dt, np.signedinteger) \
        else a.astype(np.uint64)
    with np.errstate(over="ignore"):
        ref = np.concatenate([np.zeros(1, np.uint64), np.cumsum(conv, dtype=np.uint64)[:-1]])
    np.testing.assert_array_equal(got, ref.astype(out_dt))


M48 = (1 << 48) - 1
M32 = 0xFFFFFFFF


def _py_gen(name, state):
    """Pure-Python restatement of one generator step per .cl file."""
    if name == "lcg":
        s = (state * 0x5DEECE66D + 0xB) & M48
        return s, s >> 16
    if name == "xorshift64":
        s = state
        s ^= (s << 21) & 0xFFFFFFFFFFFFFFFF
        s ^= s >> 35
        s ^= (s << 4) & 0xFFFFFFFFFFFFFFFF
        return s, s & M32
    if name == "xorshift128":
        x, y, z, w = state
        t = (x ^ (x << 11)) & M32
        w2 = (w ^ (w >> 19) ^ (t ^ (t >> 8))) & M32
        return (y, z, w, w2), w2
    if name == "mwc64x":
        x, c = state
        res = x ^ c
        hi = (x * 4294883355) >> 32
        x2 = (x * 4294883355 + c) & M32
        c2 = (hi + (1 if x2 < c else 0)) & M32
        return (x2, c2), res
    if name == "parkmiller":
        p = state * 16807
        q = abs(p) % 2147483647
        v = q if p >= 0 else -q  # C truncating remainder
        return v, ((v & M32) << 1) & M32
    if name == "tauslcg":
        x, y, z, w = state

        def taus(zz, s1, s2, s3, m):
            b = ((((zz << s1) & M32) ^ zz) >> s2)
            return ((((zz & m) << s3) & M32) ^ b)
        nx = taus(y, 13, 19, 12, 4294967294)
        ny = taus(z, 2, 25, 4, 4294967288)
        nz = taus(w, 3, 11, 17, 4294967294)
        nw = (1664525 * x + 1013904223) & M32
        return (nx, ny, nz, nw), nx
    raise ValueError(name)


def _decode(name, raw, i):
    size = oracle.SEED_SIZE[name]
    b = raw[i * size:(i + 1) * size]
    if name in ("lcg", "xorshift64"):
        return int(b.view(np.uint64)[0])
    if name == "parkmiller":
        return int(b.view(np.int32)[0])
    return tuple(int(x) for x in b.view(np.uint32))


@pytest.mark.parametrize("name", list(oracle.GEN))
def test_rng_oracle_matches_python_restatement(name):
    count, draws = 37, 5
    for hk in (0, 1, 2):
        st = oracle.rng_init_gid(name, count, 1234, hk)
        out, st2 = oracle.rng_fill(name, st, count, draws)
        for i in range(count):
            x = (i + 1234) & 0xFFFFFFFFFFFFFFFF
            if hk == 1:
                x = (x * 2654435761) % 0x100000000
            elif hk == 2:
                for _ in range(2):
                    x = (((x >> 16) ^ x) * 0x45d9f3b) & 0xFFFFFFFFFFFFFFFF
                x = (x >> 16) ^ x
            s = _decode(name, st, i)
            if name in ("lcg", "xorshift64"):
                assert s == x
            for r in range(draws):
                s, v = _py_gen(name, s)
                assert int(out[r * count + i]) == v, (name, hk, i, r)


def test_rng_fill_bits_and_maxint():
    st = oracle.rng_init_gid("lcg", 16, 7, 0)
    full, _ = oracle.rng_fill("lcg", st, 16, 3, 32, 0)
    top, _ = oracle.rng_fill("lcg", st, 16, 3, 8, 0)
    mod, _ = oracle.rng_fill("lcg", st, 16, 3, 32, 1000)
    np.testing.assert_array_equal(top, full >> 24)
    np.testing.assert_array_equal(mod, full % 1000)


def test_segmented_oracle_matches_per_segment_numpy():
    from inputs import lognormal_lengths, offsets_of, keys_of_type
    lens = lognormal_lengths(300, 5.0, 2.0, 0, 20000, seed=3)
    off = offsets_of(lens, start=4)
    n = int(off[-1]) + 5
    a = keys_of_type(8, n, np.uint32)
    got = oracle.seg_sort(a, off)
    ref = a.copy()
    for i in range(len(lens)):
        lo, hi = int(off[i]), int(off[i + 1])
        ref[lo:hi] = np.sort(a[lo:hi], kind="stable")
    np.testing.assert_array_equal(got, ref)
    v = (a >> np.uint32(24)).astype(np.uint32)
    out = oracle.seg_scan(v, off, 5, np.uint64)
    ref = np.zeros(n, np.uint64)
    for i in range(len(lens)):
        lo, hi = int(off[i]), int(off[i + 1])
        if hi > lo:
            c = np.cumsum(v[lo:hi].astype(np.uint64))
            ref[lo:hi] = np.concatenate([np.zeros(1, np.uint64), c[:-1]])
    np.testing.assert_array_equal(out, ref)

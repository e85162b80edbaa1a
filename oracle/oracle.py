"""TEST INFRASTRUCTURE -- ctypes binding of the C oracle (clo_oracle.c).

Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline
leg, as the checker. numpy arrays in, numpy arrays out.
"""
import ctypes as C
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import build_oracle  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = C.CDLL(str(path))
        P, SZ = C.c_void_p, C.c_size_t
        _lib.oracle_radix_sort.argtypes = [P, P, SZ, C.c_int, C.c_int, C.c_int]
        _lib.oracle_bitonic_sort.argtypes = [P, SZ, C.c_int]
        _lib.oracle_bitonic_sort_threaded.argtypes = [P, SZ, C.c_int, C.c_int]
        _lib.oracle_gselect_sort.argtypes = [P, P, SZ, C.c_int, P, P, C.c_int]
        _lib.oracle_scan.argtypes = [P, P, SZ, C.c_int, C.c_int]
        _lib.oracle_rng_init_gid.argtypes = [P, SZ, C.c_int, C.c_uint64, C.c_int]
        _lib.oracle_rng_fill.argtypes = [P, SZ, C.c_int, P, SZ, C.c_uint, C.c_uint]
        _lib.oracle_mt19937.argtypes = [C.c_uint32, P, SZ]
        _lib.oracle_splitmix64.argtypes = [C.c_uint64, P, SZ]
        _lib.oracle_radix_sort_u32_threaded.argtypes = [P, SZ, C.c_int, C.c_int]
        _lib.oracle_seg_sort.argtypes = [P, P, SZ, C.c_int, C.c_int]
        _lib.oracle_seg_scan.argtypes = [P, P, P, SZ, C.c_int, C.c_int]
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def radix_sort(keys, vals=None, sort_bits=None):
    k = np.ascontiguousarray(keys).copy()
    v = None if vals is None else np.ascontiguousarray(vals).copy()
    kb = k.dtype.itemsize
    vb = 0 if v is None else v.dtype.itemsize
    lib().oracle_radix_sort(_p(k), _p(v), k.size, kb, vb,
                            8 * kb if sort_bits is None else sort_bits)
    return k if v is None else (k, v)


def radix_sort_u32_threaded(keys, threads, bits=4):
    """In place on `keys` (a uint32 array); returns it."""
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    lib().oracle_radix_sort_u32_threaded(_p(k), k.size, threads, bits)
    return k


def seg_sort(keys, offsets, sort_bits=None):
    """Each segment [offsets[i], offsets[i+1]) sorted on its own (a copy)."""
    k = np.ascontiguousarray(keys).copy()
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    kb = k.dtype.itemsize
    lib().oracle_seg_sort(_p(k), _p(off), off.size - 1, kb,
                          8 * kb if sort_bits is None else sort_bits)
    return k


def seg_scan(a, offsets, in_type, out_dtype, out_init=None):
    """Per-segment exclusive scan; elements outside the segments keep
    out_init (zeros by default)."""
    a = np.ascontiguousarray(a)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    out = np.zeros(a.size, dtype=out_dtype) if out_init is None else \
        np.ascontiguousarray(out_init, dtype=out_dtype).copy()
    lib().oracle_seg_scan(_p(a), _p(out), _p(off), off.size - 1, in_type,
                          out.dtype.itemsize)
    return out


def bitonic_sort(a, clo_type):
    d = np.ascontiguousarray(a).copy()
    lib().oracle_bitonic_sort(_p(d), d.size, clo_type)
    return d


def bitonic_sort_threaded(a, clo_type, threads=None):
    """bitonic_sort's network replayed by host threads (same result)."""
    import os
    d = np.ascontiguousarray(a).copy()
    lib().oracle_bitonic_sort_threaded(_p(d), d.size, clo_type,
                                       threads or os.cpu_count() or 1)
    return d


def gselect_sort(a, clo_type, vals=None):
    a = np.ascontiguousarray(a)
    out = np.empty_like(a)
    vout = None if vals is None else np.empty_like(vals)
    lib().oracle_gselect_sort(_p(a), _p(out), a.size, clo_type,
                              _p(vals), _p(vout), 0 if vals is None else vals.dtype.itemsize)
    return out if vals is None else (out, vout)


def scan(a, in_type, out_dtype):
    a = np.ascontiguousarray(a)
    out = np.empty(a.size, dtype=out_dtype)
    lib().oracle_scan(_p(a), _p(out), a.size, in_type, out.dtype.itemsize)
    return out


GEN = {"lcg": 0, "xorshift64": 1, "xorshift128": 2, "mwc64x": 3, "parkmiller": 4,
       "tauslcg": 5}
SEED_SIZE = {"lcg": 8, "xorshift64": 8, "xorshift128": 16, "mwc64x": 8,
             "parkmiller": 4, "tauslcg": 16}


def rng_init_gid(name, count, main_seed, hash_kind=0):
    st = np.zeros(count * SEED_SIZE[name], dtype=np.uint8)
    lib().oracle_rng_init_gid(_p(st), count, GEN[name], main_seed, hash_kind)
    return st


def rng_fill(name, states, count, draws, bits=32, maxint=0):
    st = np.ascontiguousarray(states).copy()
    out = np.empty(draws * count, dtype=np.uint32)
    lib().oracle_rng_fill(_p(st), count, GEN[name], _p(out), draws, bits, maxint)
    return out, st


def mt19937(seed, nwords):
    out = np.empty(nwords, dtype=np.uint32)
    lib().oracle_mt19937(seed & 0xFFFFFFFF, _p(out), nwords)
    return out


def splitmix64(seed, n):
    out = np.empty(n, dtype=np.uint64)
    lib().oracle_splitmix64(seed, _p(out), n)
    return out


# ---- custom compare / get_key (small sizes, numpy) ----------------------
# The reference builds its kernels with CLO_SORT_COMPARE(a, b) and
# CLO_SORT_KEY_GET(x) macros (src/cl_ops/sort/clo_sort_abstract.c:141-179);
# here they are numpy callables: key_fn(elements) -> keys (already of the
# key type) and cmp_fn(k1, k2) -> bool array.

def custom_satradix(a, key_fn, key_dtype):
    """Stable sort by the key's low 8*min(element, key) bytes bits, as the
    unsigned pattern (clo_sort_satradix.c:167-169, clo_sort_satradix.cl:58,140)."""
    a = np.ascontiguousarray(a)
    k = np.ascontiguousarray(key_fn(a)).astype(key_dtype)
    kb = np.dtype(key_dtype).itemsize
    bits = 8 * min(a.dtype.itemsize, kb)
    u = k.view(f"u{kb}").astype(np.uint64)
    if bits < 64:
        u = u & np.uint64((1 << bits) - 1)
    return a[np.argsort(u, kind="stable")]


def custom_bitonic(a, key_fn, cmp_fn):
    """The reference network (clo_sort_sbitonic.c:86-108,
    clo_sort_sbitonic.cl:38-69) over the next power of two; positions past
    the elements compare greater than every element and equal to each
    other."""
    a = np.ascontiguousarray(a)
    n = a.size
    if n < 2:
        return a.copy()
    N = 1
    while N < n:
        N <<= 1
    d = np.concatenate([a, np.zeros(N - n, dtype=a.dtype)])
    pad = np.concatenate([np.zeros(n, bool), np.ones(N - n, bool)])
    g = np.arange(N // 2, dtype=np.int64)
    stages = N.bit_length() - 1
    for stage in range(1, stages + 1):
        desc = ((g >> (stage - 1)) & 1).astype(bool)
        for step in range(stage, 0, -1):
            s = 1 << (step - 1)
            i1 = g + (g // s) * s
            i2 = i1 + s
            p1, p2 = pad[i1], pad[i2]
            real = ~(p1 | p2)
            gt = p1 & ~p2
            if real.any():
                gt = gt.copy()
                gt[real] = np.asarray(cmp_fn(key_fn(d[i1[real]]), key_fn(d[i2[real]])), bool)
            sw = gt ^ desc
            x1, x2 = d[i1[sw]].copy(), d[i2[sw]].copy()
            d[i1[sw]], d[i2[sw]] = x2, x1
            q1, q2 = pad[i1[sw]].copy(), pad[i2[sw]].copy()
            pad[i1[sw]], pad[i2[sw]] = q2, q1
    return d[:n]


def custom_gselect(a, key_fn, cmp_fn):
    """out[#{i : COMPARE(k_g, k_i) or (k_i == k_g and i < g)}] = a[g]
    (clo_sort_gselect.cl:38-57)."""
    a = np.ascontiguousarray(a)
    n = a.size
    k = key_fn(a)
    out = np.empty_like(a)
    idx = np.arange(n)
    for g in range(n):
        c = np.asarray(cmp_fn(np.full(n, k[g]), k), bool)
        pos = int(np.count_nonzero(c | ((k == k[g]) & (idx < g))))
        out[pos] = a[g]
    return out

"""TEST INFRASTRUCTURE -- ctypes binding of oracle/_ref/libcloref.so, the
reference's own OpenCL kernels run on host cores (built by build_ref.py
from the reference tree). Available only where that tree is; callers
skip without it. numpy arrays in, numpy arrays out."""
import ctypes as C
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import build_ref  # noqa: E402

HASHES = build_ref.HASHES
RNGS = build_ref.RNGS
_lib = None


def available():
    return lib() is not None


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None or not path.exists():
            return None
        _lib = C.CDLL(str(path))
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"reference kernel run failed ({what}, rc={rc})")


CUSTOM = build_ref.CUSTOM


def sort(a, code, algo, lws=256, custom=None):
    """algo: 'satradix' (radix 16), 'sbitonic' or 'gselect'; returns a sorted
    copy. custom: index into CUSTOM for a sorter built with those macros."""
    d = np.ascontiguousarray(a).copy()
    f = getattr(lib(), f"ref_sort_{code}" if custom is None else f"ref_sort_c{custom}")
    f.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_size_t]
    _check(f({"satradix": 0, "sbitonic": 1, "gselect": 2}[algo], _p(d), d.size, lws),
           algo)
    return d


def scan(a, in_code, sum_code, sum_dtype, lws=128):
    a = np.ascontiguousarray(a)
    out = np.zeros(a.size, dtype=sum_dtype)
    f = getattr(lib(), f"ref_scan_{in_code}_{sum_code}")
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t]
    _check(f(_p(a), _p(out), a.size, lws), "blelloch")
    return out


SEED_SIZE = {"lcg": 8, "xorshift64": 8, "xorshift128": 16, "mwc64x": 8,
             "parkmiller": 4, "tauslcg": 16}


def rng_init(name, count, main_seed, hash_index):
    gi = RNGS.index(name)
    st = np.zeros(count * SEED_SIZE[name], dtype=np.uint8)
    f = getattr(lib(), f"ref_rng_init_{gi}")
    f.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_uint64]
    _check(f(hash_index, _p(st), count, main_seed), "rng init")
    return st


def rng_bench(name, states, count, draws, bits=32, maxint=False):
    """Returns (draws x count uint32, draw-major; states after)."""
    gi = RNGS.index(name)
    st = np.ascontiguousarray(states).copy()
    out = np.zeros(draws * count, dtype=np.uint32)
    f = getattr(lib(), f"ref_rng_bench_{gi}")
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_uint, C.c_int]
    _check(f(_p(st), count, _p(out), draws, bits, 1 if maxint else 0), "rng bench")
    return out, st

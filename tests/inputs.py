"""Seeded synthetic inputs shared by the tests and the benchmark.

splitmix64 streams (the generator named for the workloads), keys taken
from the high bits of each output; the adversarial distributions of the
large-size configuration (sorted, reverse, all-equal, 16 distinct, Zipf,
64-bit keys with only the low 20 bits varying).
"""
import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed, n, offset=0):
    """Vectorised splitmix64: output i is mix(seed + (offset + i + 1) * golden)."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def keys_u32(seed, n):
    return (splitmix64(seed, n) >> np.uint64(32)).astype(np.uint32)


def keys_u64(seed, n):
    return splitmix64(seed, n)


def keys_of_type(seed, n, np_dtype):
    raw = splitmix64(seed, n)
    size = np.dtype(np_dtype).itemsize
    if np.issubdtype(np_dtype, np.floating):
        if size == 2:
            v = (raw >> np.uint64(40)).astype(np.float64) / float(1 << 24) * 2000.0 - 1000.0
        else:
            v = (raw >> np.uint64(11)).astype(np.float64) / float(1 << 53) * 2e6 - 1e6
        return v.astype(np_dtype)
    return (raw >> np.uint64(64 - 8 * size)).astype(np.uint64).astype(
        np.dtype(f"u{size}")).view(np_dtype)


def adversarial_u32(kind, n, seed=47):
    if kind == "sorted":
        return np.sort(keys_u32(seed, n))
    if kind == "reverse":
        return np.sort(keys_u32(seed, n))[::-1].copy()
    if kind == "equal":
        return np.full(n, 0x9E3779B9, dtype=np.uint32)
    if kind == "distinct16":
        vals = keys_u32(seed + 1000, 16)
        return vals[(splitmix64(seed, n) >> np.uint64(60)).astype(np.int64)]
    if kind == "zipf":
        return zipf_u32(n, seed)
    raise ValueError(kind)


def zipf_u32(n, seed, s=1.1, ranks=1 << 20):
    """Zipf(s) over `ranks` ranks by inverse CDF; rank r maps to
    key = hi32(splitmix64(r))."""
    w = 1.0 / np.power(np.arange(1, ranks + 1, dtype=np.float64), s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    r = np.searchsorted(cdf, u, side="right")
    r = np.minimum(r, ranks - 1).astype(np.uint64)
    with np.errstate(over="ignore"):
        z = r * _G + _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(32)).astype(np.uint32)


def low20_u64(n, seed=47):
    return splitmix64(seed, n) & np.uint64((1 << 20) - 1)


def lognormal_lengths(nseg, mu, sigma, lo, hi, seed=48):
    """Segment lengths: lognormal(mu, sigma) from splitmix64 uniforms
    (Box-Muller), rounded and clipped to [lo, hi]."""
    u = (splitmix64(seed, 2 * nseg) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    u1 = np.maximum(u[0::2], 1e-300)
    u2 = u[1::2]
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    ln = np.rint(np.exp(mu + sigma * z))
    return np.clip(ln, lo, hi).astype(np.uint64)


def offsets_of(lengths, start=0):
    off = np.zeros(len(lengths) + 1, dtype=np.uint64)
    off[1:] = np.cumsum(np.asarray(lengths, dtype=np.uint64))
    return off + np.uint64(start)

"""Loads the reference known answers (tests/golden/reference_kats.json) and
regenerates each one's input."""
import hashlib
import json
import pathlib

import numpy as np

from inputs import keys_of_type

NP = {0: np.int8, 1: np.uint8, 2: np.int16, 3: np.uint16, 4: np.int32, 5: np.uint32,
      6: np.int64, 7: np.uint64, 9: np.float32, 10: np.float64}
KATS = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json")
                  .read_text())["kats"]


def select(op, **kw):
    return [k for k in KATS if k["op"] == op and all(k.get(a) == b for a, b in kw.items())]


def kat_id(k):
    keys = ("op", "algo", "code", "in", "sum", "rng", "hash", "n", "count", "bits", "maxint",
            "lws")
    return "-".join(str(k[x]) for x in keys if x in k)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sort_input(k):
    return keys_of_type(k["seed"], k["n"], NP[k["code"]])


def scan_input(k):
    return keys_of_type(k["seed"], k["n"], NP[k["in"]])


def hash_eval(text, x):
    """Value of the seed after the DEV_GID hash text (macro body applied to
    the 64-bit seed variable x), for the texts the known answers use."""
    M = 0xFFFFFFFFFFFFFFFF
    if text in ("x", "(x * 3 + 1)"):   # expressions without assignment
        return x
    if text == "KNUTH(x)":
        return (x * 2654435761) % 0x100000000
    if text == "XS1(x)":
        for _ in range(2):
            x = (((x >> 16) ^ x) * 0x45d9f3b) & M
        return (x >> 16) ^ x
    if text == "x = x << 2":
        return (x << 2) & M
    if text == "x ^= 0xABCDEF; x = x * 3 + (x >> 7) % 11":
        x ^= 0xABCDEF
        return (x * 3 + (x >> 7) % 11) & M
    raise ValueError(text)


def state_bytes(name, s):
    M = 0xFFFFFFFF
    if name in ("lcg", "xorshift64", "mwc64x"):
        return np.array([s], dtype=np.uint64).view(np.uint8)
    if name == "xorshift128":
        return np.array([s & M, (s >> 16) & M, (s >> 32) & M, (s >> 46) & M],
                        dtype=np.uint32).view(np.uint8)
    if name == "parkmiller":
        return np.array([s & M], dtype=np.uint32).view(np.uint8)
    if name == "tauslcg":
        return np.array([s, s], dtype=np.uint64).view(np.uint8)
    raise ValueError(name)


# numpy forms of the custom macros of the known answers (oracle/build_ref.py
# CUSTOM, same order): custom index -> (key_fn, cmp_fn, key dtype).
def _low32(x):
    return np.asarray(x).astype(np.uint32)


CUSTOM_FNS = {
    0: (lambda x: x, lambda a, b: a < b, np.uint32),
    1: (lambda x: x, lambda a, b: a < b, np.int32),
    2: (lambda x: x & np.uint32(0xF), lambda a, b: a > b, np.uint32),
    3: (lambda x: x >> np.uint32(4), lambda a, b: a < b, np.uint32),
    4: (_low32, lambda a, b: a > b, np.uint32),
    5: (lambda x: x, lambda a, b: a < b, np.float32),
}

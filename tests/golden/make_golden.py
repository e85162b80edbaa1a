"""Generates tests/golden/reference_kats.json: known answers computed by
the reference's own OpenCL kernels (oracle/ref.py: the cl_ops .cl files
run on host cores through oracle/ref_shim/), as SHA-256 digests of the
output bytes plus the first values. Inputs are regenerated by the tests
from the recorded generator, seed and size (tests/inputs.py).

Run from the repository root where the reference tree is available:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "oracle"), str(ROOT / "tests")]
import ref  # noqa: E402
from inputs import keys_of_type  # noqa: E402

NP = {0: np.int8, 1: np.uint8, 2: np.int16, 3: np.uint16, 4: np.int32, 5: np.uint32,
      6: np.int64, 7: np.uint64, 9: np.float32, 10: np.float64}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def head(a):
    return [x.item() for x in np.ascontiguousarray(a)[:4]]


def main():
    kats = []
    # The small radix configuration exactly as the benchmark names it:
    # 2^20 uint32 keys from splitmix64 seed 42, radix 16, keys only.
    out = ref.sort(keys_of_type(42, 1 << 20, np.uint32), 5, "satradix", 256)
    kats.append({"op": "sort", "algo": "satradix", "code": 5, "n": 1 << 20, "seed": 42,
                 "lws": 256, "config": "2^20 uint32, seed 42, radix 16",
                 "sha256": digest(out), "head": head(out)})
    for code in [0, 1, 2, 3, 4, 5, 6, 7]:
        for n, lws in [(1 << 10, 256), (1 << 12, 64), (1 << 14, 256)]:
            seed = 500 + code * 10 + n.bit_length()
            out = ref.sort(keys_of_type(seed, n, NP[code]), code, "satradix", lws)
            kats.append({"op": "sort", "algo": "satradix", "code": code, "n": n, "seed": seed,
                         "lws": lws, "sha256": digest(out), "head": head(out)})
    for code in [0, 1, 2, 3, 4, 5, 6, 7, 9, 10]:
        for n in [1 << 10, 1 << 13]:
            seed = 600 + code * 10 + n.bit_length()
            out = ref.sort(keys_of_type(seed, n, NP[code]), code, "sbitonic", 256)
            kats.append({"op": "sort", "algo": "sbitonic", "code": code, "n": n, "seed": seed,
                         "lws": 256, "sha256": digest(out), "head": head(out)})
        for n in [1000, 1 << 11]:
            seed = 700 + code * 10 + n.bit_length()
            out = ref.sort(keys_of_type(seed, n, NP[code]), code, "gselect")
            kats.append({"op": "sort", "algo": "gselect", "code": code, "n": n, "seed": seed,
                         "lws": 1, "sha256": digest(out), "head": head(out)})
    for i, (code, key, cmp, get_key) in enumerate(ref.CUSTOM):
        # satradix with a key narrower than the element is not defined in
        # the reference: its histogram shifts the untruncated element
        # (clo_sort_satradix.cl:139-140) while its local sort shifts the
        # key (:56-58), so the two disagree from the key's width on and the
        # scatter writes out of bounds.
        narrow = NP[key]().itemsize < NP[code]().itemsize
        algos = ["sbitonic", "gselect"] + (["satradix"] if code < 8 and not narrow else [])
        for algo in algos:
            n = 1000 if algo == "gselect" else 1 << 12
            seed = 900 + 10 * i + len(algo)
            out = ref.sort(keys_of_type(seed, n, NP[code]), code, algo,
                           1 if algo == "gselect" else 256, custom=i)
            kats.append({"op": "sort_custom", "custom": i, "algo": algo, "code": code,
                         "key": key, "compare": cmp, "get_key": get_key, "n": n,
                         "seed": seed, "sha256": digest(out), "head": head(out)})
    for e, s in build_pairs():
        for n, lws in [(1 << 12, 64), (1 << 16, 128), (1 << 18, 256)]:
            seed = 800 + e * 10 + s
            out = ref.scan(keys_of_type(seed, n, NP[e]), e, s, NP[s], lws)
            kats.append({"op": "scan", "in": e, "sum": s, "n": n, "seed": seed, "lws": lws,
                         "sha256": digest(out), "head": head(out)})
    for name in ref.RNGS:
        for h, text in enumerate(ref.HASHES):
            for count, main_seed in [(1000, 1234), (10000, 1234)] if h == 1 else [(1000, 1234)]:
                st = ref.rng_init(name, count, main_seed, h)
                kats.append({"op": "rng_init", "rng": name, "hash": text, "count": count,
                             "main_seed": main_seed, "sha256": digest(st)})
        st = ref.rng_init(name, 1000, 77, 3)
        for bits, maxint in [(32, False), (7, False), (1000, True)]:
            out, st2 = ref.rng_bench(name, st, 1000, 8, bits, maxint)
            kats.append({"op": "rng_bench", "rng": name, "hash": ref.HASHES[3], "count": 1000,
                         "main_seed": 77, "draws": 8, "bits": 0 if maxint else bits,
                         "maxint": bits if maxint else 0, "sha256": digest(out),
                         "states_sha256": digest(st2), "head": head(out)})
    path = pathlib.Path(__file__).with_name("reference_kats.json")
    path.write_text(json.dumps({"source": "reference OpenCL kernels on host cores "
                                          "(oracle/build_ref.py + oracle/ref_shim)",
                                "kats": kats}, indent=1) + "\n")
    print(path, len(kats))


def build_pairs():
    import build_ref
    return build_ref.SCAN_PAIRS


if __name__ == "__main__":
    main()

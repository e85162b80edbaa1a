"""Pins the CPU oracle to the reference: every known answer in
tests/golden/reference_kats.json (outputs of the reference's own OpenCL
kernels, run on host cores) is reproduced by the oracle's restatement."""
import numpy as np
import pytest

import oracle
from kats import KATS, NP, digest, hash_eval, kat_id, scan_input, select, sort_input, state_bytes


def test_kats_cover_every_path():
    ops = {(k["op"], k.get("algo")) for k in KATS}
    assert {("sort", "satradix"), ("sort", "sbitonic"), ("sort", "gselect"), ("scan", None),
            ("rng_init", None), ("rng_bench", None)} <= ops
    assert {k["rng"] for k in select("rng_bench")} == set(oracle.GEN)


@pytest.mark.parametrize("k", select("sort"), ids=kat_id)
def test_oracle_sorts_match_reference(k):
    a = sort_input(k)
    if k["algo"] == "satradix":
        out = oracle.radix_sort(a)
    elif k["algo"] == "sbitonic":
        out = oracle.bitonic_sort(a, k["code"])
    else:
        out = oracle.gselect_sort(a, k["code"])
    assert digest(out) == k["sha256"]
    assert [x.item() for x in out[:4]] == k["head"]


@pytest.mark.parametrize("k", select("scan"), ids=kat_id)
def test_oracle_scan_matches_reference(k):
    out = oracle.scan(scan_input(k), k["in"], NP[k["sum"]])
    assert digest(out) == k["sha256"]


@pytest.mark.parametrize("k", select("rng_init"), ids=kat_id)
def test_oracle_rng_seeding_matches_reference(k):
    kind = {"x": 0, "(x * 3 + 1)": 0, "KNUTH(x)": 1, "XS1(x)": 2}.get(k["hash"])
    if kind is not None:
        st = oracle.rng_init_gid(k["rng"], k["count"], k["main_seed"], kind)
    else:
        st = np.concatenate([state_bytes(k["rng"], hash_eval(k["hash"], i + k["main_seed"]))
                             for i in range(k["count"])])
    assert digest(st) == k["sha256"]


@pytest.mark.parametrize("k", select("rng_bench"), ids=kat_id)
def test_oracle_rng_draws_match_reference(k):
    st = oracle.rng_init_gid(k["rng"], k["count"], k["main_seed"], 2)
    out, st2 = oracle.rng_fill(k["rng"], st, k["count"], k["draws"], k["bits"] or 32,
                               k["maxint"])
    assert digest(out) == k["sha256"] and digest(st2) == k["states_sha256"]


@pytest.mark.parametrize("k", select("sort_custom"), ids=lambda k: f"c{k['custom']}-{k['algo']}")
def test_oracle_custom_macros_match_reference(k):
    from kats import CUSTOM_FNS
    key_fn, cmp_fn, kdt = CUSTOM_FNS[k["custom"]]
    a = sort_input(k)
    if k["algo"] == "satradix":
        out = oracle.custom_satradix(a, key_fn, kdt)
    elif k["algo"] == "sbitonic":
        out = oracle.custom_bitonic(a, key_fn, cmp_fn)
    else:
        out = oracle.custom_gselect(a, key_fn, cmp_fn)
    assert digest(out) == k["sha256"]

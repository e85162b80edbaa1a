"""The CUDA path reproduces the reference's known answers (outputs of the
reference's own OpenCL kernels, tests/golden/reference_kats.json) through
the C-ABI: every sorter (abitonic must give sbitonic's network output),
the scan, DEV_GID seeding with each hash text and the draw loop."""
import pytest

from kats import NP, digest, kat_id, scan_input, select, sort_input

pytestmark = pytest.mark.gpu


def _sort(clops, ctx, q, algo, code, a):
    s = clops.Sorter(ctx, algo, code)
    b = clops.Buffer.from_array(ctx, q, a)
    clops.wait(s.sort_device(q, b, a.size))
    out = b.read(q, a.dtype, a.size)
    b.destroy()
    s.destroy()
    return out


@pytest.mark.parametrize("k", select("sort"), ids=kat_id)
def test_cuda_sorts_match_reference(clops, ctx, queue, k):
    a = sort_input(k)
    algos = ["sbitonic", "abitonic"] if k["algo"] == "sbitonic" else [k["algo"]]
    for algo in algos:
        assert digest(_sort(clops, ctx, queue, algo, k["code"], a)) == k["sha256"], algo


@pytest.mark.parametrize("k", select("scan"), ids=kat_id)
def test_cuda_scan_matches_reference(clops, ctx, queue, k):
    a = scan_input(k)
    sc = clops.Scanner(ctx, k["in"], k["sum"])
    bi = clops.Buffer.from_array(ctx, queue, a)
    bo = clops.Buffer(ctx, a.size * NP[k["sum"]]().itemsize)
    clops.wait(sc.scan_device(queue, bi, bo, a.size))
    assert digest(bo.read(queue, NP[k["sum"]], a.size)) == k["sha256"]
    for x in (bi, bo, sc):
        x.destroy()


@pytest.mark.parametrize("k", select("rng_init"), ids=kat_id)
def test_cuda_rng_seeding_matches_reference(clops, ctx, queue, k):
    rng = clops.Rng(ctx, queue, k["rng"], clops.CLO_RNG_SEED_DEV_GID, k["count"],
                    k["main_seed"], k["hash"])
    assert digest(rng.states(queue)) == k["sha256"]
    rng.destroy()


@pytest.mark.parametrize("k", select("rng_bench"), ids=kat_id)
def test_cuda_rng_draws_match_reference(clops, ctx, queue, k):
    import numpy as np
    rng = clops.Rng(ctx, queue, k["rng"], clops.CLO_RNG_SEED_DEV_GID, k["count"],
                    k["main_seed"], k["hash"])
    out = clops.Buffer(ctx, k["count"] * k["draws"] * 4)
    clops.wait(rng.fill(queue, out, k["draws"], k["bits"] or 32, k["maxint"]))
    assert digest(out.read(queue, np.uint32, k["count"] * k["draws"])) == k["sha256"]
    assert digest(rng.states(queue)) == k["states_sha256"]
    out.destroy()
    rng.destroy()


@pytest.mark.parametrize("k", select("sort_custom"), ids=lambda k: f"c{k['custom']}-{k['algo']}")
def test_cuda_custom_macros_match_reference(clops, ctx, queue, k):
    a = sort_input(k)
    algos = ["sbitonic", "abitonic"] if k["algo"] == "sbitonic" else [k["algo"]]
    for algo in algos:
        s = clops.Sorter(ctx, algo, k["code"], key_type=k["key"], compare=k["compare"],
                         get_key=k["get_key"])
        b = clops.Buffer.from_array(ctx, queue, a)
        clops.wait(s.sort_device(queue, b, a.size))
        assert digest(b.read(queue, a.dtype, a.size)) == k["sha256"], algo
        b.destroy()
        s.destroy()

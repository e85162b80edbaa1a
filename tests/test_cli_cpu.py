"""The benchmark programs (ports of the reference's clo_sort_bench,
clo_scan_bench and clo_rng_bench command lines): option tables and
argument errors, without a GPU."""
import pathlib
import subprocess

import pytest

BIN = pathlib.Path(__file__).resolve().parents[1] / "cl-ops_gb300" / "bin"
CLO_ERROR_ARGS = 2


def run(name, *args):
    exe = BIN / name
    if not exe.exists():
        pytest.skip("benchmark programs not built")
    return subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("name,opts", [
    ("clo_sort_bench", ["--algorithm", "--alg-opts", "--runs", "--localsize", "--device",
                        "--rng-seed", "--type", "--maxpo2", "--out", "--compiler"]),
    ("clo_scan_bench", ["--runs", "--localsize", "--device", "--rng-seed", "--type",
                        "--type-sum", "--init-elems", "--num-doub", "--compiler",
                        "--algorithm", "--alg-opts", "--no-check", "--out"]),
    ("clo_rng_bench", ["--rng", "--output", "--globalsize", "--localsize", "--runs",
                       "--device", "--rng-seed", "--gid-hash", "--bits", "--max"]),
])
def test_help_lists_the_reference_options(name, opts):
    r = run(name, "--help")
    assert r.returncode == 0
    for o in opts:
        assert o in r.stdout, o


@pytest.mark.parametrize("name,args", [
    ("clo_sort_bench", ["--bogus"]),
    ("clo_scan_bench", ["-x"]),
    ("clo_rng_bench", ["--bits", "33"]),
    ("clo_rng_bench", ["--output", "nowhere"]),
    ("clo_rng_bench", ["--runs", "0", "--output", "file-tsv"]),
    ("clo_sort_bench", ["--maxpo2"]),
])
def test_argument_errors(name, args):
    r = run(name, *args)
    assert r.returncode == CLO_ERROR_ARGS
    assert "Error" in r.stderr

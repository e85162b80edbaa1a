"""The benchmark programs on the GPU: sorted and scanned outputs verified
by the programs' own checks, and random numbers equal to the oracle's."""
import pathlib
import re
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
BIN = pathlib.Path(__file__).resolve().parents[1] / "cl-ops_gb300" / "bin"


def run(name, *args, cwd=None):
    exe = BIN / name
    if not exe.exists():
        pytest.skip("benchmark programs not built")
    return subprocess.run([str(exe), *args], capture_output=True, cwd=cwd, timeout=300)


@pytest.mark.parametrize("algo,typ", [("satradix", "uint"), ("abitonic", "int"),
                                      ("sbitonic", "double"), ("gselect", "uchar")])
def test_sort_bench_sorts(algo, typ, tmp_path):
    maxpo2 = "12" if algo == "gselect" else "16"
    r = run("clo_sort_bench", "-a", algo, "-t", typ, "-n", maxpo2, "-r", "2", "-o",
            str(tmp_path / "s.tsv"))
    out = r.stdout.decode()
    assert r.returncode == 0, r.stderr
    lines = re.findall(r"- 2\^(\d+): ([0-9.]+) Mkeys/s(.*)", out)
    assert [int(x[0]) for x in lines] == list(range(4, int(maxpo2) + 1))
    assert all(x[2].strip() == "" for x in lines)  # no "(sort did not work)"
    rows = (tmp_path / "s.tsv").read_text().splitlines()
    assert len(rows) == int(maxpo2) and all(len(r.split("\t")) == 3 for r in rows)


def test_scan_bench_checks(tmp_path):
    r = run("clo_scan_bench", "-n", "16", "-r", "2", "-t", "uint", "-y", "ulong")
    assert r.returncode == 0, r.stderr
    out = r.stdout.decode()
    assert out.count("MValues/s") == 16 and "did not work" not in out


@pytest.mark.parametrize("name", ["lcg", "mwc64x", "parkmiller", "xorshift128"])
def test_rng_bench_outputs_match_oracle(name, tmp_path):
    gws, runs = 1000, 3
    r = run("clo_rng_bench", "-r", name, "-g", str(gws), "-n", str(runs), "-h", "XS1(x)",
            "-b", "20", "-o", "file-tsv", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    f = tmp_path / f"out_{name}_gid_XS1(x).tsv"
    got = np.array([[int(v) for v in line.rstrip("\t").split("\t")]
                    for line in f.read_text().splitlines()], dtype=np.uint32)
    st = oracle.rng_init_gid(name, gws, 0, 2)
    exp, _ = oracle.rng_fill(name, st, gws, runs, 20)
    np.testing.assert_array_equal(got.reshape(-1), exp)
    r = run("clo_rng_bench", "-r", name, "-g", str(gws), "-n", "2", "-o", "stdout-bin",
            "-m", "1000")
    raw = np.frombuffer(r.stdout, dtype=np.uint32)
    assert raw.size == 2 * gws and raw.max() < 1000

"""TEST INFRASTRUCTURE -- builds oracle/_ref/libcloref.so: the reference's
own OpenCL kernels (cl_ops .cl files, read where they lie in the reference
tree) compiled as host C++ through the shim in oracle/ref_shim/, with host
drivers that restate the reference's launch sequences.

Nothing of the reference is copied into the repository: the kernel text
is read at build time, rewritten mechanically (OpenCL qualifiers removed,
vector literals turned into constructor calls, work-group-local
declarations given per-thread static storage) and written only under
oracle/_ref/ (git-ignored). The generated units stay in oracle/_ref/gen/,
so a machine without the reference tree that received a copy of them
(a checkout copied together with its git-ignored build outputs) compiles
them as they are. With neither, the build is skipped and the callers skip
the live comparisons; the committed known-answer digests (tests/golden/)
were produced from this library.

Usage: python oracle/build_ref.py [--force] [--reference DIR]
Reference location: --reference, else $CLO_REFERENCE_ROOT, else the
directory named "reference" beside the repository checkout.
"""
import concurrent.futures as cf
import os
import pathlib
import re
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
SHIM = HERE / "ref_shim"
OUT = HERE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libcloref.so"

# CloType code -> OpenCL type name as the reference prints it
# (clo_type_get_name) and the host type it means here.
TYPES = {0: ("char", "schar"), 1: ("uchar", "uchar"), 2: ("short", "short"),
         3: ("ushort", "ushort"), 4: ("int", "int"), 5: ("uint", "uint"),
         6: ("long", "long"), 7: ("ulong", "ulong"), 9: ("float", "float"),
         10: ("double", "double")}
SORT_INT = [0, 1, 2, 3, 4, 5, 6, 7]
SORT_ALL = SORT_INT + [9, 10]
SCAN_PAIRS = [(5, 7), (5, 5), (0, 4), (1, 5), (2, 6), (4, 4), (7, 7), (6, 6), (3, 3),
              (0, 0)]
RNGS = ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller", "tauslcg"]
# DEV_GID hashes, in the order of ref.HASHES.
HASHES = ["x", "(x * 3 + 1)", "KNUTH(x)", "XS1(x)", "x = x << 2",
          "x ^= 0xABCDEF; x = x * 3 + (x >> 7) % 11"]
SATRADIX_BITS = 4  # the reference's default radix 16
# Sorters built with custom macros: (element code, key code, compare,
# get_key), as a caller of clo_sort_new would pass them.
CUSTOM = [(5, 5, "((a) < (b))", "(x)"),
          (4, 4, "((a) < (b))", "(x)"),
          (5, 5, "((a) > (b))", "((x) & 0xF)"),
          (5, 5, "((a) < (b))", "((x) >> 4)"),
          (7, 5, "((a) > (b))", "(x)"),
          (9, 9, "((a) < (b))", "(x)")]


_ROOT_OVERRIDE = None


def ref_root():
    if _ROOT_OVERRIDE is not None:
        return pathlib.Path(_ROOT_OVERRIDE)
    env = os.environ.get("CLO_REFERENCE_ROOT")
    return pathlib.Path(env) if env else HERE.parent.parent / "reference"


def to_cxx(text):
    """OpenCL C kernel text -> C++ for clc_host.h."""
    out = []
    for line in text.splitlines():
        s = line.strip()
        if re.match(r"__local\b.*;\s*$", s) and "(" not in s.split("__local", 1)[0]:
            line = line.replace("__local", "static thread_local", 1)
        line = re.sub(r"\b__(kernel|global|local|constant)\b", "", line)
        line = re.sub(r"\((uint2|uint4|uint8|ulong2|clo_statetype)\)\s*\(", r"\1(", line)
        out.append(line)
    return "\n".join(out) + "\n"


def cl(rel):
    return to_cxx((ref_root() / rel).read_text())


def unit_sort(code, key=None, compare="((a) > (b))", get_key="(x)", tag=None):
    cname, hname = TYPES[code]
    kname = TYPES[code if key is None else key][1]
    tag = str(code) if tag is None else tag
    scan = cl("src/cl_ops/scan/clo_scan_blelloch.cl")
    srcs = [cl("src/cl_ops/sort/clo_sort_sbitonic.cl"), cl("src/cl_ops/sort/clo_sort_gselect.cl")]
    if code in SORT_INT:
        srcs.insert(0, cl("src/cl_ops/sort/clo_sort_satradix.cl"))
    body = [
        '#include "clc_host.h"', "#include <vector>", f"namespace ns_sort_{tag} {{",
        "namespace scan {", "#define CLO_SCAN_ELEM_TYPE uint", "#define CLO_SCAN_SUM_TYPE uint",
        scan, '#include "drv_scan.inc"', "#undef CLO_SCAN_ELEM_TYPE", "#undef CLO_SCAN_SUM_TYPE",
        "}",
        f"#define CLO_SORT_ELEM_TYPE {hname}", f"#define CLO_SORT_KEY_TYPE {kname}",
        f"#define CLO_SORT_COMPARE(a, b) {compare}", f"#define CLO_SORT_KEY_GET(x) {get_key}",
        f"#define CLO_SORT_NUM_BITS {SATRADIX_BITS}",
    ] + srcs
    if code in SORT_INT:
        body.append('#include "drv_sort.inc"')
    else:
        body.append('#define CLC_NO_SATRADIX\n#include "drv_sort.inc"')
    body += ["}",
             f'extern "C" int ref_sort_{tag}(int algo, void *data, size_t n, size_t lws) {{',
             f"  using namespace ns_sort_{tag};"]
    if code in SORT_INT:
        body.append("  if (algo == 0) return drive_satradix(data, n, lws) ? 0 : -1;")
    body += ["  if (algo == 1) return drive_sbitonic(data, n, lws) ? 0 : -1;",
             "  if (algo == 2) return drive_gselect(data, n) ? 0 : -1;", "  return -2;", "}"]
    return "\n".join(body)


def unit_scan(e, s):
    body = ['#include "clc_host.h"', "#include <vector>", f"namespace ns_scan_{e}_{s} {{",
            f"#define CLO_SCAN_ELEM_TYPE {TYPES[e][1]}", f"#define CLO_SCAN_SUM_TYPE {TYPES[s][1]}",
            cl("src/cl_ops/scan/clo_scan_blelloch.cl"), '#include "drv_scan.inc"', "}",
            f'extern "C" int ref_scan_{e}_{s}(const void *in, void *out, size_t n, size_t lws) {{',
            f"  return ns_scan_{e}_{s}::drive_scan(in, out, n, lws) ? 0 : -1;", "}"]
    return "\n".join(body)


def unit_rng(gi, name):
    gen = cl(f"src/cl_ops/rng/clo_rng_{name}.cl")
    wi = cl("src/cl_ops/rng/clo_rng_workitem.cl")
    api = cl("src/cl_ops/rng/clo_rng_api.cl")
    init = cl("src/cl_ops/rng/clo_rng_init.cl")
    bench = cl("src/benchmarks/clo_rng_bench.cl")
    body = ['#include "clc_host.h"', "#include <vector>", f"namespace ns_rng_{gi} {{",
            gen, wi, api]
    for h, text in enumerate(HASHES):
        body += [f"namespace h{h} {{", "#undef CLO_RNG_HASH",
                 f"#define CLO_RNG_HASH(x) {text}", init, "}"]
    body += [bench, "namespace mx {", "#define CLO_RNG_BENCHMARK_MAXINT", bench,
             "#undef CLO_RNG_BENCHMARK_MAXINT", "}", '#include "drv_rng.inc"', "}",
             f'extern "C" int ref_rng_init_{gi}(int hash, void *states, size_t count, ulong main_seed) {{',
             f"  using namespace ns_rng_{gi};", "  bool ok = false;", "  switch (hash) {"]
    for h in range(len(HASHES)):
        body.append(f"  case {h}: ok = clc_run(count, 1, [&] {{ h{h}::clo_rng_init(main_seed, "
                    f"(clo_statetype *)states); }}); break;")
    body += ["  default: return -2;", "  }", "  return ok ? 0 : -1;", "}",
             f'extern "C" int ref_rng_bench_{gi}(void *states, size_t count, uint *out, '
             "size_t draws, uint bits, int maxint) {",
             f"  return ns_rng_{gi}::drive_bench(states, count, out, draws, bits, maxint != 0) ? 0 : -1;",
             "}"]
    return "\n".join(body)


def units():
    u = {f"sort_{c}": unit_sort(c) for c in SORT_ALL}
    u.update({f"sort_c{i}": unit_sort(e, k, cmp, key, tag=f"c{i}")
              for i, (e, k, cmp, key) in enumerate(CUSTOM)})
    u.update({f"scan_{e}_{s}": unit_scan(e, s) for e, s in SCAN_PAIRS})
    u.update({f"rng_{i}": unit_rng(i, n) for i, n in enumerate(RNGS)})
    return u


def build(force=False):
    """Returns the library path, or None without the reference tree and
    without previously generated units."""
    if (ref_root() / "src" / "cl_ops").is_dir():
        GEN.mkdir(parents=True, exist_ok=True)
        srcs = []
        for name, text in units().items():
            p = GEN / f"{name}.cpp"
            if not p.exists() or p.read_text() != text:
                p.write_text(text)
            srcs.append(p)
    else:
        srcs = sorted(GEN.glob("*.cpp")) if GEN.is_dir() else []
        if not srcs:
            return LIB if LIB.exists() else None
    srcs.append(SHIM / "clc_runner.cpp")
    shim_time = max(q.stat().st_mtime for q in SHIM.iterdir())
    if LIB.exists() and not force and all(
            LIB.stat().st_mtime > max(q.stat().st_mtime, shim_time) for q in srcs):
        return LIB
    cxx = shutil.which("g++") or "g++"
    flags = ["-O1", "-std=c++17", "-fPIC", "-pthread", "-w", f"-I{SHIM}"]

    def comp(src):
        obj = GEN / (src.stem + ".o")
        subprocess.run([cxx, *flags, "-c", str(src), "-o", str(obj)], check=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(comp, srcs))
    subprocess.run([cxx, "-shared", "-pthread", "-o", str(LIB), *map(str, objs)], check=True)
    return LIB


if __name__ == "__main__":
    if "--reference" in sys.argv:
        _ROOT_OVERRIDE = sys.argv[sys.argv.index("--reference") + 1]
    print(build(force="--force" in sys.argv))

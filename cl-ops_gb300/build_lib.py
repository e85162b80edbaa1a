"""Builds libclops.so (the C-ABI library: host layer + sm_103a kernels).

Usage: python build_lib.py [--force]

Every translation unit is compiled by nvcc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, into _build/, and
linked with the CUDA runtime statically so the library has no loader-path
dependency. Objects are rebuilt only when a source or header is newer.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
INCLUDE = ROOT / "include"
BUILD = HERE / "_build"
LIB = HERE / "libclops.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", f"-I{INCLUDE}", f"-I{CSRC}",
          "-Xcompiler", "-fPIC,-Wall",
          "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def gen_rng_source() -> None:
    """Embeds include/clo_rng_device.cuh as a C string (the text that
    clo_rng_get_source returns)."""
    text = (INCLUDE / "clo_rng_device.cuh").read_text()
    esc = text.replace("\\", "\\\\").replace('"', '\\"')
    body = "\n".join('"%s\\n"' % line for line in esc.split("\n"))
    out = "static const char kRngDeviceSource[] =\n" + body + ";\n"
    dst = CSRC / "_gen_rng_device_src.inc"
    if not dst.exists() or dst.read_text() != out:
        dst.write_text(out)


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def newest_header() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list(CSRC.glob("*.inc")) + list(INCLUDE.glob("*.h")) + \
        list(INCLUDE.glob("*.cuh"))
    return max(p.stat().st_mtime for p in hs)


def compile_one(src: pathlib.Path, force: bool, hdr_time: float):
    obj = BUILD / (src.name + ".o")
    if not force and obj.exists():
        t = obj.stat().st_mtime
        if t >= src.stat().st_mtime and t >= hdr_time:
            return obj, None
    cmd = [nvcc()] + ARCH + COMMON + ["-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "cu"] + ARCH + COMMON + ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    gen_rng_source()
    hdr = newest_header()
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: compile_one(s, force, hdr), srcs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("compilation failed:\n" + "\n".join(errors))
    objs = [str(o) for o, _ in results]
    if force or not LIB.exists() or LIB.stat().st_mtime < max(
            pathlib.Path(o).stat().st_mtime for o in objs):
        # Export only the C ABI (clo_* and ccl_* symbols).
        vs = BUILD / "exports.map"
        vs.write_text("{ global: clo_*; ccl_*; local: *; };\n")
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", str(LIB)] + \
            objs + ["-lrt", "-ldl", "-lpthread", "-Xlinker", f"--version-script={vs}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    build_cli(force)
    if verbose:
        print(f"built {LIB}")
    return LIB


CLI = HERE / "cli"
BIN = HERE / "bin"


def build_cli(force: bool = False) -> None:
    """The benchmark programs (cli/*.c) against libclops.so, into bin/."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        return
    BIN.mkdir(exist_ok=True)
    hdr = max(p.stat().st_mtime for p in list(CLI.glob("*.h")) + list(INCLUDE.glob("*.h")))
    for src in sorted(CLI.glob("*.c")):
        exe = BIN / src.stem
        if not force and exe.exists() and exe.stat().st_mtime >= max(
                src.stat().st_mtime, hdr, LIB.stat().st_mtime):
            continue
        cmd = [cc, "-O2", "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-Wall", f"-I{INCLUDE}",
               f"-I{CLI}", str(src), "-o", str(exe), f"-L{HERE}", "-lclops",
               "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)

"""TEST INFRASTRUCTURE -- builds the CPU oracle (clo_oracle.c) into
oracle/_build/libclo_oracle.so with the host C compiler."""
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build" / "libclo_oracle.so"


def build(force: bool = False) -> pathlib.Path:
    src = HERE / "clo_oracle.c"
    hdr = HERE / "clo_oracle.h"
    OUT.parent.mkdir(exist_ok=True)
    if (not force and OUT.exists()
            and OUT.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return OUT
    cc = shutil.which("gcc") or shutil.which("cc")
    cmd = [cc, "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", "-Wall",
           str(src), "-o", str(OUT), "-lm"]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force=True))

"""Build the host-core chi0 kernel of the CPU path (oracle/cpu_chi0.cpp) into oracle/_build/.

Test and measurement infrastructure only: g++ with OpenMP, no architecture flags, so the same
source builds on x86-64 and on aarch64.  Rebuilds when the source is newer than the library.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_chi0.cpp"
OUT = HERE / "_build" / "libcpu_chi0.so"


def build() -> Path:
    if OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the CPU path")
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    r = subprocess.run([cxx, "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", str(SRC), "-o", str(tmp)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building {SRC.name} failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build())

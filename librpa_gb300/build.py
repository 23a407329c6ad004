"""Build the GB300 RPA shared library in-tree (no cmake).

Compiles every translation unit of csrc/ for sm_103a with nvcc, in parallel,
and links librpa_gb300/liblibrpa_gb300.so.  Object files go to
librpa_gb300/_build/.  Rebuilds only what changed (source or header mtime).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
SRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblibrpa_gb300.so"
DRIVER_SRC = PKG / "driver" / "chi0_main.cpp"
DRIVER = PKG / "chi0_main"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
          "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted([p for p in SRC.iterdir() if p.suffix in (".cu", ".cpp")])


def _stale(src: Path, obj: Path, headers_mtime: float) -> bool:
    if not obj.exists():
        return True
    m = obj.stat().st_mtime
    return src.stat().st_mtime > m or headers_mtime > m


def build(verbose: bool = False, jobs: int | None = None, extra: list[str] | None = None) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    hdrs = list(SRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    hmt = max((h.stat().st_mtime for h in hdrs), default=0.0)
    srcs = sources()
    objs = [BUILD / (s.name + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if _stale(s, o, hmt)]

    def compile_one(so):
        s, o = so
        cmd = [nvcc, *ARCH, *CFLAGS, *(extra or []), "-x", "cu" if s.suffix == ".cu" else "c++", "-c", str(s), "-o", str(o)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return s.name

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for name in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", name)
    if todo or not LIB.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_driver(hmt)
    return LIB


def build_driver(headers_mtime: float = 0.0) -> Path:
    """The task = rpa driver executable (host C++ over the C API), linked to the library."""
    if DRIVER.exists() and DRIVER.stat().st_mtime > max(DRIVER_SRC.stat().st_mtime, LIB.stat().st_mtime,
                                                         headers_mtime):
        return DRIVER
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(DRIVER_SRC), "-L", str(PKG),
           "-l:liblibrpa_gb300.so", "-Wl,-rpath,$ORIGIN", "-o", str(DRIVER)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

"""The C++ interface include/librpa.hpp (the reference's include/librpa.hpp), compiled against
this library: option defaults, errors as exceptions, and on a GB300 the E_c of the C API."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def exe(lib, tmp_path_factory):
    from librpa_gb300.build import LIB, PKG
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("hpp") / "hpp_wrapper"
    subprocess.run([cxx, "-O1", "-std=c++17", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "hpp_wrapper.cpp"), "-L", str(PKG), "-l:" + LIB.name,
                    f"-Wl,-rpath,{PKG}", "-o", str(out)], check=True)
    return out


def test_wrapper_without_gpu(exe, lib):
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test covers the full run")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK no-gpu" in r.stdout


@pytest.mark.gpu
def test_wrapper_ec_equals_c_api(exe):
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK gpu" in r.stdout

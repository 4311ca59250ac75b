"""The C++ adapter a maintainer adds to the reference (include/AmrDG_GB300.h),
compiled against a stand-in for the AMReX interface it uses
(tests/cxx/amrex_standin.h) and linked to the library:

* CPU: the adapter and the compiled test build with g++ (syntax and types).
* GPU: the compiled test steps a three-level hierarchy held in per-(level, q)
  FArrayBox-style device arrays through the zero-copy patch boundary
  (adg_set_patches / adg_read_patches / adg_write_patches) and checks it
  bit for bit against a context stepping its own packed state.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CXX_DIR = os.path.join(ROOT, "tests", "cxx")
SRC = os.path.join(CXX_DIR, "test_amrdg_gb300.cpp")
LIB_DIR = os.path.join(ROOT, "ader-dg-amr_gb300", "adg_gb300", "_lib")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _cxx():
    c = shutil.which("g++") or shutil.which("c++")
    if not c:
        pytest.skip("no C++ compiler")
    return c


def _flags():
    return ["-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", CXX_DIR,
            "-I", os.path.join(CUDA, "include")]


def test_adapter_compiles_against_the_amrex_interface():
    r = subprocess.run([_cxx(), *_flags(), "-fsyntax-only", SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_adapter_steps_caller_arrays_bit_for_bit(tmp_path):
    import adg_gb300  # noqa: F401  (the library must be built)

    exe = str(tmp_path / "test_amrdg_gb300")
    libcuda = os.path.join(CUDA, "lib64")
    cmd = [_cxx(), *_flags(), SRC, "-o", exe, "-L", LIB_DIR, "-ladg", "-L", libcuda, "-lcudart",
           f"-Wl,-rpath,{LIB_DIR}", f"-Wl,-rpath,{libcuda}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")

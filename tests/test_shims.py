"""The cu:: shims (include/cu_gb300_shims.hpp) build: against the reference's own
linalg::CsrMatrix<float> header where the reference tree is present (syntax check of every shim
class instantiated with it), and the reference-shaped time-step loop program tests/shims/chorin_loop.cpp
compiles and links against the library.  No GPU needed; tests/test_gpu_shims.py runs the program."""

import os
import shutil
import subprocess

import pytest

from conftest import ROOT

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


def build_loop(out_dir):
    """Compile and link tests/shims/chorin_loop.cpp against libnsfem_gb300.so; returns the program."""
    from nsfemoptim_gb300 import _build
    lib_dir = os.path.dirname(_build.LIB)
    out = os.path.join(out_dir, "chorin_loop")
    cmd = [NVCC, "-std=c++17", "-O2", os.path.join(ROOT, "tests", "shims", "chorin_loop.cpp"),
           "-I", os.path.join(ROOT, "include"), "-L" + lib_dir, "-lnsfem_gb300", "-Xlinker", "-rpath," + lib_dir,
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_loop_program_builds(tmp_path):
    if not os.path.exists(NVCC):
        pytest.skip("nvcc not found")
    import nsfemoptim_gb300  # noqa: F401  (the library is built)
    assert os.path.exists(build_loop(str(tmp_path)))


def test_shims_compile_against_reference_csr_matrix():
    import oracle
    root = oracle.reference_root()
    inc = os.path.join(root, "libs", "LinAlg", "include") if root else ""
    if not inc or not os.path.isdir(inc):
        pytest.skip("reference tree not present")
    gxx = shutil.which("g++")
    cmd = [gxx, "-std=c++20", "-fsyntax-only", "-I", inc, "-I", os.path.join(root, "libs", "Utils", "include"),
           "-I", os.path.join(ROOT, "include"), "-I",
           "/usr/local/cuda/include", os.path.join(ROOT, "tests", "shims", "reference_types.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

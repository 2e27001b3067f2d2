"""In-tree build of libnsfem_gb300.so: the sm_103a CUDA kernels and C ABI (nvcc) plus the C++ host
setup (g++), linked into one shared library next to this file.  Used by ``__graft_entry__.build()``
and on first import when the library is missing.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnsfem_gb300.so")
CLI = os.path.join(HERE, "nsf_solver_test")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["host/mesh.cpp", "host/context.cpp", "host/io.cpp"]
CUDA_SOURCES = ["capi.cu"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cuh", ".h", ".hpp"))]
    headers.append(os.path.join(CSRC, "host", "setup.hpp"))
    headers.append(os.path.join(HERE, "..", "include", "nsfem_gb300.h"))
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([NVCC, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out, file=sys.stderr)
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs])
    # the SolverTest-compatible command-line tool, over the C ABI of the library
    cli_src = os.path.join(HERE, "cli", "solver_test.cpp")
    if force or _newer(CLI, [cli_src, LIB, os.path.join(HERE, "..", "include", "nsfem_gb300.h")]):
        _run(["g++", "-std=c++17", "-O2", "-Wall", cli_src, "-o", CLI, "-L" + HERE, "-lnsfem_gb300",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))

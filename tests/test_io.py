"""Binary CSR / vector interchange files (nsf_io_*) against the reference's own reader and writer
(cpp/libs/LinAlg/src/io.cpp, compiled into the reference harness), and the SolverTest-compatible
command-line tool's argument handling.  No GPU needed.

* Round trips through the C ABI keep every integer and every value (FP64 files) or the FP32 rounding
  (FP32 files).
* Files written here are byte-identical to the files the reference writes for the same data, and
  each side reads the other's files: live where the reference harness is built, and everywhere
  through SHA-256 digests of the reference's files for the committed 33 x 33 square's P1 Laplacian
  and a seeded vector (tests/golden/ref_io_square_n33.json, written by tests/golden/make_golden.py).
* Malformed files fail with NSF_ERR_IO, as the reference's reader throws.
"""

import ctypes as C
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def G():
    import nsfemoptim_gb300 as G
    return G


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _laplacian(square_small, O):
    import scipy.sparse as sp

    from nsfemoptim_gb300 import meshgen
    m = O.Mesh(square_small)
    rs, ci, val = meshgen.p1_stiffness(m.corner_xy.astype(np.float64), m.tri)
    K = sp.csr_matrix((val, ci, rs))
    K.sort_indices()
    return K.indptr.astype(np.int32), K.indices.astype(np.int32), K.data.astype(np.float64), K.shape[0]


def _write_csr(G, path, rs, ci, v, n, dtype):
    L = G.lib()
    assert L.nsf_io_write_csr(path.encode(), n, n, len(ci), _p(rs, C.c_int), _p(ci, C.c_int), _p(v, C.c_double),
                              dtype) == 0, L.nsf_last_error()


def _read_csr(G, path):
    L = G.lib()
    info = (C.c_int * 4)()
    st = L.nsf_io_csr_info(path.encode(), info)
    if st != 0:
        return st, None
    rows, cols, nnz, dt = list(info)
    rs = np.zeros(rows + 1, np.int32)
    ci = np.zeros(nnz, np.int32)
    v = np.zeros(nnz)
    assert L.nsf_io_read_csr(path.encode(), _p(rs, C.c_int), _p(ci, C.c_int), _p(v, C.c_double)) == 0
    return 0, (rows, cols, dt, rs, ci, v)


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


@pytest.mark.parametrize("dtype", [0, 1])
def test_csr_and_vector_roundtrip(G, oracle_lib, square_small, tmp_path, dtype):
    rs, ci, v, n = _laplacian(square_small, oracle_lib)
    path = str(tmp_path / "a.csr")
    _write_csr(G, path, rs, ci, v, n, dtype)
    st, (rows, cols, dt, rs2, ci2, v2) = _read_csr(G, path)
    assert st == 0 and (rows, cols, dt) == (n, n, dtype)
    assert np.array_equal(rs, rs2) and np.array_equal(ci, ci2)
    assert np.array_equal(v2, v if dtype == 1 else v.astype(np.float32).astype(np.float64))
    x = np.random.default_rng(2).standard_normal(n)
    vp = str(tmp_path / "x.vec")
    L = G.lib()
    assert L.nsf_io_write_vec(vp.encode(), n, _p(x, C.c_double), dtype) == 0
    info = (C.c_int * 2)()
    assert L.nsf_io_vec_info(vp.encode(), info) == 0 and list(info) == [n, dtype]
    y = np.zeros(n)
    assert L.nsf_io_read_vec(vp.encode(), _p(y, C.c_double)) == 0
    assert np.array_equal(y, x if dtype == 1 else x.astype(np.float32).astype(np.float64))


def test_malformed_files_rejected(G, tmp_path):
    L = G.lib()
    info = (C.c_int * 4)()
    bad = tmp_path / "bad.csr"
    bad.write_bytes(np.array([7, 2, 2, 1], np.int32).tobytes())  # unknown dtype id
    assert L.nsf_io_csr_info(str(bad).encode(), info) == 6
    bad.write_bytes(np.array([1, 2, 2, 3], np.int32).tobytes() + np.zeros(3).tobytes())  # data cut short
    assert L.nsf_io_csr_info(str(bad).encode(), info) == 6
    # rowStart[rows] != nnz
    body = np.array([1, 2, 2, 2], np.int32).tobytes() + np.ones(2).tobytes() + np.array([0, 1], np.int32).tobytes() + \
        np.array([0, 1, 1], np.int32).tobytes()
    bad.write_bytes(body)
    assert L.nsf_io_csr_info(str(bad).encode(), info) == 6
    assert L.nsf_io_csr_info(str(tmp_path / "missing.csr").encode(), info) == 6
    vec = tmp_path / "bad.vec"
    vec.write_bytes(np.array([0, 0], np.int32).tobytes())  # n < 1
    assert L.nsf_io_vec_info(str(vec).encode(), (C.c_int * 2)()) == 6


def _golden_io():
    with open(os.path.join(GOLDEN, "ref_io_square_n33.json")) as f:
        return json.load(f)


def test_files_match_golden_reference_digests(G, oracle_lib, square_small, tmp_path):
    """Ours writes, for the committed square's Laplacian and the seeded vector, the bytes that the
    reference's linalg::write wrote (its SHA-256 digests, per dtype)."""
    g = _golden_io()
    rs, ci, v, n = _laplacian(square_small, oracle_lib)
    x = np.random.default_rng(g["vector_seed"]).standard_normal(n)
    L = G.lib()
    for dtype in (0, 1):
        path = str(tmp_path / f"a{dtype}.csr")
        _write_csr(G, path, rs, ci, v, n, dtype)
        assert _sha(path) == g["csr_sha256"][str(dtype)]
        vp = str(tmp_path / f"x{dtype}.vec")
        assert L.nsf_io_write_vec(vp.encode(), n, _p(x, C.c_double), dtype) == 0
        assert _sha(vp) == g["vec_sha256"][str(dtype)]


def test_files_match_live_reference(G, oracle_lib, square_small, tmp_path):
    """Each side reads the other's files; equal bytes for equal data."""
    R = oracle_lib.reference()
    if R is None:
        pytest.skip("reference harness (oracle/_ref) not built on this machine")
    O = oracle_lib
    rs, ci, v, n = _laplacian(square_small, O)
    x = np.random.default_rng(3).standard_normal(n)
    for dtype in (0, 1):
        ours, theirs = str(tmp_path / f"o{dtype}.csr"), str(tmp_path / f"r{dtype}.csr")
        _write_csr(G, ours, rs, ci, v, n, dtype)
        assert R.ref_io_write_csr(theirs.encode(), dtype, n, n, len(ci), O._ptr(rs, C.c_int), O._ptr(ci, C.c_int),
                                  O._ptr(v, C.c_double)) == 0
        assert _sha(ours) == _sha(theirs)
        st, (rows, cols, dt, rs2, ci2, v2) = _read_csr(G, theirs)
        assert st == 0 and np.array_equal(rs2, rs) and np.array_equal(ci2, ci)
        dims = (C.c_int * 3)()
        rr = np.zeros(n + 1, np.int32)
        cc = np.zeros(len(ci), np.int32)
        vv = np.zeros(len(ci))
        assert R.ref_io_read_csr(ours.encode(), dtype, dims, O._ptr(rr, C.c_int), O._ptr(cc, C.c_int),
                                 O._ptr(vv, C.c_double)) == 0
        assert np.array_equal(rr, rs) and np.array_equal(cc, ci) and np.array_equal(vv, v2)
        ov, rv = str(tmp_path / f"o{dtype}.vec"), str(tmp_path / f"r{dtype}.vec")
        assert G.lib().nsf_io_write_vec(ov.encode(), n, _p(x, C.c_double), dtype) == 0
        assert R.ref_io_write_vec(rv.encode(), dtype, n, O._ptr(x, C.c_double)) == 0
        assert _sha(ov) == _sha(rv)


def _cli():
    from nsfemoptim_gb300 import _build
    return _build.CLI


def test_cli_arguments(G, tmp_path):
    """The command line of the reference's SolverTest; its CPU algorithms are named as not provided;
    unreadable input fails before any device work."""
    cli = _cli()
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "<algo> <matrix> <rhs>" in r.stderr
    r = subprocess.run([cli, "cgCuda", str(tmp_path / "none.csr"), str(tmp_path / "none.vec")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "failed to open" in r.stderr
    # a 2 x 2 system: the header lines print, then the algorithm is checked
    rs = np.array([0, 1, 2], np.int32)
    ci = np.array([0, 1], np.int32)
    v = np.array([2.0, 4.0])
    m, b = str(tmp_path / "m.csr"), str(tmp_path / "b.vec")
    _write_csr(G, m, rs, ci, v, 2, 0)
    bb = np.array([1.0, 1.0])
    assert G.lib().nsf_io_write_vec(b.encode(), 2, _p(bb, C.c_double), 0) == 0
    r = subprocess.run([cli, "jacobi", m, b], capture_output=True, text=True)
    assert r.returncode == 1 and "Matrix size = 2x2" in r.stdout and "Number of channels = 1" in r.stdout
    assert "CPU algorithms" in r.stderr
    r = subprocess.run([cli, "nosuch", m, b], capture_output=True, text=True)
    assert r.returncode == 1 and "No algorithm matching nosuch" in r.stderr

"""Regenerate the golden fixtures of tests/golden.

1. Synthetic meshes (seeded, written by nsfemoptim_gb300.meshgen) are stored gzipped:
   channel_h0.025_s0.msh.gz (DFG channel, h = 0.025) and square_n33_s0.msh.gz (jittered unit square).
2. The reference's own C++ (oracle/_ref/libnsfref.so, built from the reference sources by
   oracle/Makefile.ref) reads those files and produces the integer structures that parity is pinned
   on: P2/P1 numbering, border elements, Dirichlet/internal lists, the CSR sparsity prototypes of
   M/K, Kp, D, G and the FastConvection integration matrix, and the smallest-last + greedy coloring
   of M and of the internal pressure stiffness.  Their SHA-256 digests (little-endian int32/float32
   bytes) and a few small arrays are written to ref_<mesh>.json.
3. The reference's element integrator (triangleIntegrator.cpp, compiled into the same harness
   against a test-only cv::Mat stand-in) gives the FP32 local matrices of 48 seeded elements of the
   channel mesh: ref_local_<mesh>.npz.
4. The reference's binary writer (linalg::write, io.cpp) writes the square's P1 Laplacian and a seeded
   vector as float and double files: their SHA-256 digests go to ref_io_square_n33.json.

Run from the repository root where the reference tree is present:
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import ctypes as C
import gzip
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nsfemoptim_gb300 import meshgen  # noqa: E402


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def ref_structures(R, path: str, peak: float) -> dict:
    h = R.ref_mesh_load(path.encode())
    if not h:
        raise RuntimeError(R.ref_last_error().decode())
    c = (C.c_int * 6)()
    R.ref_mesh_counts(h, c)
    V, T, B, N, P, ng = list(c)
    out = {"counts": {"corner": V, "triangles": T, "border": B, "N": N, "P": P},
           "groups": [R.ref_mesh_group(h, i).decode() for i in range(ng)], "sha256": {}}
    sh = out["sha256"]
    v_elem = np.zeros(6 * T, np.int32)
    R.ref_mesh_elements(h, 2, oracle._ptr(v_elem, C.c_int))
    p_elem = np.zeros(3 * T, np.int32)
    R.ref_mesh_elements(h, 1, oracle._ptr(p_elem, C.c_int))
    v_xy = np.zeros(2 * N, np.float32)
    R.ref_mesh_nodes(h, 2, oracle._ptr(v_xy, C.c_float))
    v_border = np.zeros(6 * B, np.int32)
    R.ref_mesh_border(h, 2, oracle._ptr(v_border, C.c_int))
    sh.update(v_elem=digest(v_elem), p_elem=digest(p_elem), v_xy=digest(v_xy), v_border=digest(v_border))
    if all(g in out["groups"] for g in ("Left", "Right", "Top", "Bottom", "Circle")):
        d = (C.c_int * 4)()
        R.ref_dirichlet(h, peak, d, None, None, None, None, None)
        vx = np.zeros(d[0], np.int32)
        vv = np.zeros(d[0], np.float32)
        pi = np.zeros(d[1], np.int32)
        iv = np.zeros(d[2], np.int32)
        ip = np.zeros(d[3], np.int32)
        R.ref_dirichlet(h, peak, d, oracle._ptr(vx, C.c_int), oracle._ptr(vv, C.c_float), oracle._ptr(pi, C.c_int),
                        oracle._ptr(iv, C.c_int), oracle._ptr(ip, C.c_int))
        out["peak_velocity"] = peak
        sh.update(dir_ids=digest(vx), dir_vx=digest(vv), dir_p_ids=digest(pi), int_v=digest(iv), int_p=digest(ip))
        out["dir_vx_max"] = float(vv.max())
        out["counts"].update(n_dir=int(d[0]), n_dir_p=int(d[1]))
    protos = {}
    for w, name in enumerate(["M", "Kp", "D", "G", "I"]):
        ph = R.ref_prototype(h, w)
        dims = (C.c_int * 3)()
        R.ref_csr_dims(ph, dims)
        rs = np.zeros(dims[0] + 1, np.int32)
        cl = np.zeros(dims[2], np.int32)
        R.ref_csr_arrays(ph, oracle._ptr(rs, C.c_int), oracle._ptr(cl, C.c_int), None)
        R.ref_csr_free(ph)
        protos[name] = (rs, cl)
        sh[f"{name}_rowStart"] = digest(rs)
        sh[f"{name}_col"] = digest(cl)
        out["counts"][f"nnz_{name}"] = int(dims[2])

    def color(rs, cl, tag, rows=None):
        if rows is not None:
            # internal pressure slice through the reference's CsrMatrix::slice
            ph0 = R.ref_csr_wrap(len(rs) - 1, len(rs) - 1, len(cl), oracle._ptr(rs, C.c_int), oracle._ptr(cl, C.c_int),
                                 None)
            ph = R.ref_csr_slice(ph0, len(rows), oracle._ptr(rows, C.c_int), len(rows), oracle._ptr(rows, C.c_int))
            R.ref_csr_free(ph0)
            dims = (C.c_int * 3)()
            R.ref_csr_dims(ph, dims)
            rs = np.zeros(dims[0] + 1, np.int32)
            cl = np.zeros(dims[2], np.int32)
            R.ref_csr_arrays(ph, oracle._ptr(rs, C.c_int), oracle._ptr(cl, C.c_int), None)
            sh[f"{tag}_rowStart"] = digest(rs)
            sh[f"{tag}_col"] = digest(cl)
        else:
            ph = R.ref_csr_wrap(len(rs) - 1, len(rs) - 1, len(cl), oracle._ptr(rs, C.c_int), oracle._ptr(cl, C.c_int),
                                None)
        nc = R.ref_coloring(ph, None, None, None)
        order = np.zeros(len(rs) - 1, np.int32)
        part = np.zeros(nc + 1, np.int32)
        sl = np.zeros(len(rs) - 1, np.int32)
        R.ref_coloring(ph, oracle._ptr(order, C.c_int), oracle._ptr(part, C.c_int), oracle._ptr(sl, C.c_int))
        R.ref_csr_free(ph)
        sh[f"color_{tag}_perm"] = digest(order)
        sh[f"color_{tag}_slorder"] = digest(sl)
        out[f"color_{tag}_partStart"] = part.tolist()

    color(*protos["M"], "M")
    if "int_p" in sh:
        color(*protos["Kp"], "Kpi", rows=ip)
    else:
        color(*protos["Kp"], "Kp")
    R.ref_mesh_free(h)
    return out


def ref_local_sample(R, path: str, count: int = 48, seed: int = 0) -> dict:
    """The reference integrator's local matrices (float32) for `count` seeded elements of the mesh."""
    h = R.ref_mesh_load(path.encode())
    c = (C.c_int * 6)()
    R.ref_mesh_counts(h, c)
    elems = np.sort(np.random.default_rng(seed).choice(c[1], size=count, replace=False)).astype(np.int32)
    mats = [oracle.reference_local_matrices(R, h, int(e)) for e in elems]
    R.ref_mesh_free(h)
    out = {"elements": elems}
    for k in mats[0]:
        out[k] = np.stack([m[k] for m in mats]).astype(np.float32)
    return out


def ref_io_digests(R, square_path: str, seed: int = 11) -> dict:
    """SHA-256 of the files the reference's linalg::write produces for the square's P1 Laplacian and
    a seeded N(0, 1) vector, as float (dtype 0) and double (dtype 1)."""
    import tempfile

    import scipy.sparse as sp

    m = oracle.Mesh(square_path)
    rs, ci, val = meshgen.p1_stiffness(m.corner_xy.astype(np.float64), m.tri)
    K = sp.csr_matrix((val, ci, rs))
    K.sort_indices()
    rs, ci, v = K.indptr.astype(np.int32), K.indices.astype(np.int32), K.data.astype(np.float64)
    n = K.shape[0]
    x = np.random.default_rng(seed).standard_normal(n)
    out = {"vector_seed": seed, "n": n, "nnz": int(len(ci)), "csr_sha256": {}, "vec_sha256": {}}
    with tempfile.TemporaryDirectory() as d:
        for dtype in (0, 1):
            p = os.path.join(d, "a.csr")
            assert R.ref_io_write_csr(p.encode(), dtype, n, n, len(ci), oracle._ptr(rs, C.c_int),
                                      oracle._ptr(ci, C.c_int), oracle._ptr(v, C.c_double)) == 0
            with open(p, "rb") as f:
                out["csr_sha256"][str(dtype)] = hashlib.sha256(f.read()).hexdigest()
            p = os.path.join(d, "x.vec")
            assert R.ref_io_write_vec(p.encode(), dtype, n, oracle._ptr(x, C.c_double)) == 0
            with open(p, "rb") as f:
                out["vec_sha256"][str(dtype)] = hashlib.sha256(f.read()).hexdigest()
    return out


def main():
    oracle.build()
    if not oracle.build_reference():
        raise SystemExit("the reference sources are needed to regenerate the golden structures")
    R = oracle.reference()
    meshes = {"channel_h0.025_s0": (meshgen.dfg_channel(0.025, seed=0), 1.2),
              "square_n33_s0": (meshgen.jittered_square(33, seed=0), 1.0)}
    for name, (m, peak) in meshes.items():
        raw = os.path.join(HERE, name + ".msh")
        meshgen.write_gmsh41(raw, m)
        with open(raw, "rb") as f, gzip.GzipFile(raw + ".gz", "wb", mtime=0) as g:
            g.write(f.read())
        res = ref_structures(R, raw, peak)
        if name.startswith("channel"):
            np.savez_compressed(os.path.join(HERE, f"ref_local_{name}.npz"), **ref_local_sample(R, raw))
        else:
            with open(os.path.join(HERE, "ref_io_square_n33.json"), "w") as f:
                json.dump(ref_io_digests(R, raw), f, indent=1, sort_keys=True)
        os.remove(raw)
        with open(os.path.join(HERE, f"ref_{name}.json"), "w") as f:
            json.dump(res, f, indent=1, sort_keys=True)
        print(name, res["counts"])


if __name__ == "__main__":
    main()

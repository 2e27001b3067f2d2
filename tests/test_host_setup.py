"""The product's host setup (C++ behind the C ABI) against the oracle and the reference golden
fixtures: integers bit-exact, FP64 values to 1e-14 relative.  No GPU needed."""

import ctypes as C
import hashlib
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def G():
    import nsfemoptim_gb300 as G
    return G


def test_library_exports_every_declared_symbol(G):
    with open(os.path.join(ROOT, "include", "nsfem_gb300.h")) as f:
        text = f.read()
    declared = set(re.findall(r"\b(nsf_[a-z0-9_]+)\s*\(", text))
    L = C.CDLL(G.LIB_PATH)
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    from nsfemoptim_gb300 import _lib
    assert declared == set(_lib.declared_symbols())


def test_product_matches_golden_reference_structures(G, channel_coarse):
    with open(os.path.join(GOLDEN, "ref_channel_h0.025_s0.json")) as f:
        g = json.load(f)
    m = G.load_gmsh(channel_coarse)
    assert m.groups == g["groups"]
    ve, pe, vxy, vb = m.arrays()
    sh = g["sha256"]
    assert digest(ve.ravel()) == sh["v_elem"]
    assert digest(pe.ravel()) == sh["p_elem"]
    assert digest(vxy.ravel()) == sh["v_xy"]
    assert digest(vb.ravel()) == sh["v_border"]
    ctx = G.build_chorin_context(m, g["peak_velocity"], 4)
    assert digest(ctx.dir_ids) == sh["dir_ids"]
    assert digest(ctx.dir_vx.astype(np.float32)) == sh["dir_vx"]
    assert digest(ctx.dir_p_ids) == sh["dir_p_ids"]
    assert digest(ctx.int_v) == sh["int_v"]
    assert digest(ctx.int_p) == sh["int_p"]
    for name in ("M", "Kp", "D", "G", "I"):
        a = ctx.matrix(name)
        assert digest(a.rowStart) == sh[f"{name}_rowStart"], name
        assert digest(a.column) == sh[f"{name}_col"], name
    assert digest(ctx.matrix("Kpi").rowStart) == sh["Kpi_rowStart"]
    for name, tag in (("M", "M"), ("Kpi", "Kpi")):
        a = ctx.matrix(name)
        perm, part = G.coloring(a.rowStart, a.column)
        assert digest(perm) == sh[f"color_{tag}_perm"]
        assert part.tolist() == g[f"color_{tag}_partStart"]


@pytest.mark.parametrize("threads", [1, 3])
def test_product_values_match_oracle(G, oracle_lib, channel_coarse, threads):
    O = oracle_lib
    m = G.load_gmsh(channel_coarse)
    ctx = G.build_chorin_context(m, 1.2, threads)
    oc = O.Context(O.Mesh(channel_coarse), 1.2, True)
    for name in ("M", "K", "Kp", "Kpi", "D", "G", "I"):
        a, b = ctx.matrix(name), getattr(oc, name)
        assert np.array_equal(a.rowStart, b.rowStart) and np.array_equal(a.column, b.col), name
        assert np.max(np.abs(a.values - b.val)) <= 1e-14 * np.max(np.abs(b.val)), name
    assert np.array_equal(ctx.dir_vx, oc.dir_vx)


def test_assembly_deterministic_across_threads(G, channel_coarse):
    m = G.load_gmsh(channel_coarse)
    a = G.build_chorin_context(m, 1.2, 1)
    b = G.build_chorin_context(m, 1.2, 7)
    for name in ("M", "K", "D", "G", "I"):
        assert np.array_equal(a.matrix(name).values, b.matrix(name).values), name


def test_square_mesh_matches_golden(G, square_small):
    with open(os.path.join(GOLDEN, "ref_square_n33_s0.json")) as f:
        g = json.load(f)
    m = G.load_gmsh(square_small)
    ve, pe, vxy, vb = m.arrays()
    assert digest(ve.ravel()) == g["sha256"]["v_elem"]
    ctx = G.build_chorin_context(m, 1.0, 2)
    kp = ctx.matrix("Kp")
    assert digest(kp.column) == g["sha256"]["Kp_col"]


def test_p1_stiffness_matches_context(G, square_small):
    """meshgen.p1_stiffness (the pressure-only Poisson workload's assembly) is the operator the
    context assembles as Kp: same pattern, values within the float-coordinate rounding."""
    from nsfemoptim_gb300 import meshgen
    m = G.load_gmsh(square_small)
    ve, pe, vxy, vb = m.arrays()
    # P1 node coordinates from the triangles' corners (P2 nodes 0, 2, 4)
    xy = np.zeros((m.P, 2))
    for k in range(3):
        xy[pe[:, k]] = vxy[ve[:, 2 * k]]
    rs, ci, val = meshgen.p1_stiffness(xy, pe)
    kp = G.build_chorin_context(m, 1.0, 2).matrix("Kp")
    assert np.array_equal(rs, kp.rowStart) and np.array_equal(ci, kp.column)
    assert np.abs(val - kp.values).max() <= 1e-5 * np.abs(kp.values).max()
    # a Laplacian: rows sum to zero
    assert np.abs(np.add.reduceat(val, rs[:-1])).max() < 1e-9


def test_bad_inputs_rejected_with_status(G, tmp_path):
    from nsfemoptim_gb300 import _lib
    # missing file
    with pytest.raises(G.NsfError) as e:
        G.load_gmsh(str(tmp_path / "nope.msh"))
    assert e.value.status == _lib.NSF_ERR_IO
    # truncated gmsh file
    p = tmp_path / "bad.msh"
    p.write_text("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$Nodes\n1 2 1 2\n")
    with pytest.raises(G.NsfError):
        G.load_gmsh(str(p))
    # CSR validation before upload (no GPU touched): unsorted columns, out of range, bad rowStart
    rs = np.array([0, 2, 3], np.int32)
    for col in ([1, 0, 1], [0, 5, 1]):
        with pytest.raises(G.NsfError) as e:
            G.CsrF(2, 2, rs, np.array(col, np.int32), np.ones(3))
        assert e.value.status == _lib.NSF_ERR_INVALID_ARG
    with pytest.raises(G.NsfError):
        G.CsrF(2, 2, np.array([0, 3, 2], np.int32), np.array([0, 1, 1], np.int32), np.ones(3))
    with pytest.raises(G.NsfError):
        G.CsrF(2, 2, rs, np.array([0, 1, 1], np.int32), np.array([1.0, np.nan, 1.0]))
    # coloring needs a valid pattern too
    with pytest.raises(G.NsfError):
        G.coloring(np.array([0, 2, 3], np.int32), np.array([1, 1, 0], np.int32))


def test_channel_mesh_generator_sizes():
    from nsfemoptim_gb300 import meshgen
    m = meshgen.dfg_channel(0.025, seed=0)
    p = m.nodes[m.triangles]
    det = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    assert det.min() > 0
    area = 0.5 * det.sum()
    assert abs(area - (2.2 * 0.41 - np.pi * 0.05 ** 2)) < 1e-3
    assert 3000 < m.num_triangles < 4500  # reference h = 0.025 mesh: 3,554 triangles
    assert set(m.border) == {"Right", "Top", "Left", "Bottom", "Circle"}
    # the same seed gives the same mesh
    m2 = meshgen.dfg_channel(0.025, seed=0)
    assert np.array_equal(m.nodes, m2.nodes) and np.array_equal(m.triangles, m2.triangles)


def test_async_set_state_refuses_arrays_that_need_copies(G):
    """An asynchronous state upload reads the caller's arrays after the call returns, so
    ChorinStepper.set_state refuses, before any library call, arrays that would need a temporary
    C-contiguous float64 copy; the flag values match the header's."""
    class Unbound:
        _h = None

    u = np.zeros(8)
    p = np.zeros(4)
    for bad_u, bad_p in ((u[::2], p), (u.astype(np.float32), p), (list(u), p), (u, p[::2])):
        with pytest.raises(ValueError):
            G.ChorinStepper.set_state(Unbound(), bad_u, bad_p, asynchronous=True)
    with open(os.path.join(ROOT, "include", "nsfem_gb300.h")) as f:
        text = f.read()
    assert re.search(r"#define NSF_STATE_KEEP_HISTORY 1\b", text)
    assert re.search(r"#define NSF_STATE_ASYNC 2\b", text)
    assert (G.NSF_STATE_KEEP_HISTORY, G.NSF_STATE_ASYNC) == (1, 2)

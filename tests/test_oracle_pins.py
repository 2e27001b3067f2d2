"""The oracle pinned against the reference's own code.

* Golden fixtures (tests/golden/ref_*.json): digests of integer structures that the reference's
  C++ produced from the committed synthetic meshes (tests/golden/make_golden.py).  These run
  everywhere.
* Live comparison against oracle/_ref/libnsfref.so (the reference sources compiled here) on the
  committed meshes and on the reference's own shipped meshes when the reference tree is present.
"""

import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, shipped_mesh_path


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def _golden(name):
    with open(os.path.join(GOLDEN, f"ref_{name}.json")) as f:
        return json.load(f)


def _check_against_golden(O, path, g, with_bcs):
    m = O.Mesh(path)
    assert m.groups == g["groups"]
    c = g["counts"]
    assert (m.num_corner, m.num_tri, m.num_border, m.N, m.P) == (c["corner"], c["triangles"], c["border"], c["N"],
                                                                  c["P"])
    sh = g["sha256"]
    assert digest(m.v_elem.ravel()) == sh["v_elem"]
    assert digest(m.p_elem.ravel()) == sh["p_elem"]
    assert digest(m.v_xy.ravel()) == sh["v_xy"]
    assert digest(m.v_border.ravel()) == sh["v_border"]
    ctx = O.Context(m, g.get("peak_velocity", 1.0), True)
    if with_bcs:
        assert digest(ctx.dir_ids) == sh["dir_ids"]
        assert digest(ctx.dir_vx.astype(np.float32)) == sh["dir_vx"]
        assert np.array_equal(ctx.dir_vx, ctx.dir_vx.astype(np.float32).astype(np.float64))
        assert digest(ctx.dir_p_ids) == sh["dir_p_ids"]
        assert digest(ctx.int_v) == sh["int_v"]
        assert digest(ctx.int_p) == sh["int_p"]
    for name in ("M", "Kp", "D", "G", "I"):
        a = getattr(ctx, name)
        assert digest(a.rowStart) == sh[f"{name}_rowStart"], name
        assert digest(a.col) == sh[f"{name}_col"], name
    perm, part, sl = O.coloring(ctx.M)
    assert digest(perm) == sh["color_M_perm"]
    assert digest(sl) == sh["color_M_slorder"]
    assert part.tolist() == g["color_M_partStart"]
    if with_bcs:
        assert digest(ctx.Kpi.rowStart) == sh["Kpi_rowStart"]
        assert digest(ctx.Kpi.col) == sh["Kpi_col"]
        perm, part, sl = O.coloring(ctx.Kpi)
        assert digest(perm) == sh["color_Kpi_perm"]
        assert digest(sl) == sh["color_Kpi_slorder"]
        assert part.tolist() == g["color_Kpi_partStart"]
    return m, ctx


def test_oracle_matches_reference_golden_channel(oracle_lib, channel_coarse):
    _check_against_golden(oracle_lib, channel_coarse, _golden("channel_h0.025_s0"), True)


def test_oracle_matches_reference_golden_square(oracle_lib, square_small):
    _check_against_golden(oracle_lib, square_small, _golden("square_n33_s0"), True)


def _hole_area(m, gid):
    """Area of the polygon formed by the border edges of group gid (star-shaped from (0.2, 0.2))."""
    vb = m.v_border[m.v_border[:, 2] == gid]
    a = m.v_xy.astype(np.float64)[vb[:, 3]] - (0.2, 0.2)
    b = m.v_xy.astype(np.float64)[vb[:, 5]] - (0.2, 0.2)
    return 0.5 * np.abs(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]).sum()


def test_force_functional_identities(oracle_lib, channel_coarse):
    """Drag/lift functional (new, no reference counterpart): exact for fields the elements
    represent exactly.  With n pointing into the fluid (out of the hole H):
      u = 0, p = x        ->  F = -integral(x n) = (-|H|, 0)
      u = (x^2, 0), p = 0 ->  F = nu integral(2 x n_x, 0) = (2 nu |H|, 0)"""
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    gid = m.groups.index("Circle")
    H = _hole_area(m, gid)
    n_edges = int((m.v_border[:, 2] == gid).sum())
    # inscribed regular-ish polygon of the r = 0.05 circle
    assert abs(H - 0.5 * n_edges * 0.05 ** 2 * np.sin(2 * np.pi / n_edges)) < 0.02 * H
    # pressure node coordinates: the corners of each triangle (c0, c1, c2 = P2 nodes 0, 2, 4)
    px = np.zeros(m.P)
    for t in range(m.num_tri):
        for k in range(3):
            px[m.p_elem[t, k]] = m.v_xy[m.v_elem[t, 2 * k], 0]
    f = O.forces(m, np.zeros(2 * m.N), px, 1e-3)
    assert abs(f[0] + H) < 1e-12 and abs(f[1]) < 1e-12
    # x^2 at the corners and at the exact edge midpoints (the stored midpoint coordinates are
    # float-rounded, which would perturb the interpolant at the 1e-6 level)
    u = np.zeros(2 * m.N)
    xv = m.v_xy[:, 0].astype(np.float64)
    for t in range(m.num_tri):
        c = m.v_elem[t]
        for k in (0, 2, 4):
            u[c[k]] = xv[c[k]] ** 2
        for mid, a, b in ((1, 0, 2), (3, 2, 4), (5, 4, 0)):
            u[c[mid]] = (0.5 * (xv[c[a]] + xv[c[b]])) ** 2
    nu = 2e-3
    f = O.forces(m, u, np.zeros(m.P), nu)
    assert abs(f[0] - 2 * nu * H) < 1e-12 and abs(f[1]) < 1e-12


def test_fem_identities(oracle_lib, channel_coarse):
    """Values are restated (the reference integrator needs OpenCV): check the physics instead."""
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, True)
    p = m.corner_xy.astype(np.float64)[m.tri]
    area = 0.5 * np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) -
                        (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])).sum()
    assert abs(area - (2.2 * 0.41 - np.pi * 0.05 ** 2)) < 1e-3
    # the mass matrix sums to the (polygonal) domain area (the element maps use float edge
    # vectors, as the reference's affine transforms do); stiffness rows sum to zero
    assert abs(ctx.M.val.sum() - area) < 1e-9
    ones = np.ones(ctx.N)
    assert np.max(np.abs(O.spmv(ctx.K, ones))) < 1e-11
    assert np.max(np.abs(O.spmv(ctx.Kp, np.ones(ctx.P)))) < 1e-11
    # symmetry of M, K, Kp
    for a in (ctx.M, ctx.K, ctx.Kp):
        s = a.to_scipy()
        assert abs(s - s.T).max() < 1e-14 * abs(s).max()
    # divergence of a constant field and gradient of a constant pressure vanish
    assert np.max(np.abs(O.spmv(ctx.D, np.r_[ones, np.zeros(ctx.N)]))) < 1e-12
    assert np.max(np.abs(O.spmv(ctx.G, np.ones(ctx.P)))) < 1e-12
    # D u + G^T u is a boundary term: zero for a field vanishing on the boundary
    # (integration by parts), checked with u = bubble-like interior field
    xy = m.v_xy.astype(np.float64)
    bub = xy[:, 0] * (2.2 - xy[:, 0]) * xy[:, 1] * (0.41 - xy[:, 1]) * \
        np.maximum(0, (xy[:, 0] - 0.2) ** 2 + (xy[:, 1] - 0.2) ** 2 - 0.05 ** 2)
    bub[ctx.dir_ids] = 0
    onb = np.zeros(ctx.N, bool)
    onb[ctx.dir_ids] = True
    u = np.r_[bub, 0.5 * bub]
    lhs = O.spmv(ctx.D, u)
    rhs = -ctx.G.to_scipy().T @ u
    assert np.max(np.abs(lhs[ctx.int_p] - rhs[ctx.int_p])) < 1e-9 * np.max(np.abs(lhs))
    # FastConvection: I u gives the convection values C(u); C(u) applied to a constant is zero
    rng = np.random.default_rng(0)
    uu = rng.standard_normal(2 * ctx.N)
    cvals = O.fastconv(ctx, 0.0, uu)
    c = O.Csr(ctx.K.rows, ctx.K.cols, ctx.K.rowStart, ctx.K.col, cvals)
    assert np.max(np.abs(O.spmv(c, ones))) < 1e-11 * np.max(np.abs(cvals))


def _reference():
    import oracle
    R = oracle.reference()
    if R is None:
        pytest.skip("reference harness (oracle/_ref) not built on this machine")
    return R


def _ref_meshes():
    out = []
    for name in ("h_0.025.msh", "h_0.01.msh", "h_0.005.msh"):
        p = shipped_mesh_path(name)
        if p:
            out.append(p)
    return out


@pytest.mark.parametrize("which", ["committed", "reference"])
def test_oracle_matches_live_reference(oracle_lib, channel_coarse, which):
    import ctypes as C
    R = _reference()
    O = oracle_lib
    paths = [channel_coarse] if which == "committed" else _ref_meshes()
    if not paths:
        pytest.skip("reference meshes not present")
    for path in paths:
        h = R.ref_mesh_load(path.encode())
        assert h, R.ref_last_error()
        c = (C.c_int * 6)()
        R.ref_mesh_counts(h, c)
        m = O.Mesh(path)
        assert list(c)[:5] == [m.num_corner, m.num_tri, m.num_border, m.N, m.P]
        e2 = np.zeros(6 * m.num_tri, np.int32)
        R.ref_mesh_elements(h, 2, O._ptr(e2, C.c_int))
        assert np.array_equal(e2.reshape(-1, 6), m.v_elem)
        ctx = O.Context(m, 1.2, True)
        for w, name in enumerate(["M", "Kp", "D", "G", "I"]):
            ph = R.ref_prototype(h, w)
            dims = (C.c_int * 3)()
            R.ref_csr_dims(ph, dims)
            rs = np.zeros(dims[0] + 1, np.int32)
            cl = np.zeros(dims[2], np.int32)
            R.ref_csr_arrays(ph, O._ptr(rs, C.c_int), O._ptr(cl, C.c_int), None)
            R.ref_csr_free(ph)
            a = getattr(ctx, name)
            assert np.array_equal(rs, a.rowStart) and np.array_equal(cl, a.col), name
        a = ctx.Kpi
        ph = R.ref_csr_wrap(a.rows, a.cols, a.nnz, O._ptr(a.rowStart, C.c_int), O._ptr(a.col, C.c_int), None)
        nc = R.ref_coloring(ph, None, None, None)
        order = np.zeros(a.rows, np.int32)
        part = np.zeros(nc + 1, np.int32)
        R.ref_coloring(ph, O._ptr(order, C.c_int), O._ptr(part, C.c_int), None)
        R.ref_csr_free(ph)
        perm, opart, _ = O.coloring(a)
        assert np.array_equal(order, perm) and np.array_equal(part, opart)
        R.ref_mesh_free(h)


def test_multicolor_gs_matches_reference_gs2ch(oracle_lib, channel_coarse):
    """A multicolor sweep equals a natural-order sweep of the color-permuted matrix; the reference's
    double-precision gaussSeidel2ch on that matrix pins the oracle's sweep arithmetic."""
    import ctypes as C
    R = _reference()
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, False)
    col = O.coloring(ctx.M)
    perm = col[0]
    Mp = O.slice_csr(ctx.M, perm, perm)
    n = Mp.rows
    rng = np.random.default_rng(3)
    b = rng.standard_normal(2 * n)
    x_ref = np.zeros(2 * n)
    b_inter = np.empty(2 * n)
    b_inter[0::2], b_inter[1::2] = b[:n], b[n:]
    res = np.zeros(2)
    iters = 7
    R.ref_gs2ch_double(n, O._ptr(Mp.rowStart, C.c_int), O._ptr(Mp.col, C.c_int), O._ptr(Mp.val, C.c_double),
                       O._ptr(x_ref, C.c_double), O._ptr(b_inter, C.c_double), iters, 0.0, O._ptr(res, C.c_double))
    # oracle: the same 7 sweeps in the original numbering (target 0 -> never stops early)
    b_orig = np.zeros(2 * n)
    b_orig[perm], b_orig[n + perm] = b[:n], b[n:]
    x, rms, it = O.gs_solve(ctx.M, col, 2, b_orig, np.zeros(2 * n), iters, 0.0, 1)
    xo = np.r_[x[:n][perm], x[n:][perm]]
    xr = np.r_[x_ref[0::2], x_ref[1::2]]
    assert np.max(np.abs(xo - xr)) <= 1e-13 * np.max(np.abs(xr))
    assert np.allclose(rms, res, rtol=1e-10)


def test_oracle_adjoint_matches_finite_differences(oracle_lib, channel_coarse):
    """The FP64 discrete adjoint of the oracle (no reference counterpart) against FP64 central
    differences of its own forward run: d/dnu, two inflow sine-series coefficients and a random
    direction of the initial velocity.  J = mean drag over the second half of 10 steps."""
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.0)
    nu, tau, n = 1e-3, 5e-4, 10
    wd = np.zeros(n)
    wd[n // 2:] = 1.0 / (n - n // 2)
    rng = np.random.default_rng(5)
    u0 = np.zeros(2 * ctx.N)
    u0[:ctx.N] = 0.3 * rng.random(ctx.N)
    u0[ctx.N:] = 0.05 * rng.standard_normal(ctx.N)
    J, gnu, gdir, gu = O.adjoint_run(ctx, m, nu, tau, n, wd, u0=u0)

    def fwd(nu_=nu, dv=None, uu=u0):
        s = O.Chorin(ctx, nu_, tau, vel_method=1, vel_max_iters=100000, vel_tol=1e-14, pres_max_iters=100000,
                     pres_tol=1e-14)
        s.set_state(uu, np.zeros(ctx.P))
        s.set_dirichlet(ctx.dir_vx if dv is None else dv)
        out = 0.0
        for k in range(n):
            s.step()
            if wd[k]:
                uk, pk = s.state()
                out += wd[k] * O.forces(m, uk, pk, nu_)[0]
        return out

    assert abs(fwd() - J) <= 1e-14 * abs(J)
    eps = 1e-6
    fd = (fwd(nu_=nu + eps) - fwd(nu_=nu - eps)) / (2 * eps)
    assert abs(fd - gnu) <= 1e-6 * abs(gnu)
    xy = m.v_xy.astype(np.float64)[ctx.dir_ids]
    inflow = np.abs(xy[:, 0]) < 1e-9
    # per coefficient for the two largest components; normwise over four (a small component's
    # relative error is FD noise at the solver-tolerance level divided by eps)
    fds, gs = [], []
    for k in (1, 2, 3, 4):
        b = np.where(inflow, np.sin(k * np.pi * xy[:, 1] / 0.41), 0.0)
        fds.append((fwd(dv=ctx.dir_vx + eps * b) - fwd(dv=ctx.dir_vx - eps * b)) / (2 * eps))
        gs.append(float(b @ gdir))
    fds, gs = np.array(fds), np.array(gs)
    for i in (0, 2):
        assert abs(fds[i] - gs[i]) <= 1e-6 * abs(gs[i])
    assert np.linalg.norm(fds - gs) <= 1e-6 * np.linalg.norm(gs)
    d = rng.standard_normal(2 * ctx.N)
    d[ctx.dir_ids] = 0.0
    d[ctx.N + ctx.dir_ids] = 0.0
    fd = (fwd(uu=u0 + eps * d) - fwd(uu=u0 - eps * d)) / (2 * eps)
    g = float(d @ gu)
    assert abs(fd - g) <= 1e-6 * abs(g)
    assert np.all(gu[ctx.dir_ids] == 0) and np.all(gu[ctx.N + ctx.dir_ids] == 0)


def _p2_element_mass():
    """P2 element mass matrix on one triangle (unit area): basis lambda_i (2 lambda_i - 1) at the
    vertices and 4 lambda_i lambda_j at the edge midpoints, integrated exactly with
    int lambda1^a lambda2^b lambda3^c dA = 2 |T| a! b! c! / (a + b + c + 2)!."""
    from math import factorial

    def mul(p, q):
        out = {}
        for ka, va in p.items():
            for kb, vb in q.items():
                k = tuple(x + y for x, y in zip(ka, kb))
                out[k] = out.get(k, 0.0) + va * vb
        return out

    def integrate(p):
        return sum(v * 2.0 * factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 2)
                   for (a, b, c), v in p.items())

    e = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    basis = []
    for i in range(3):
        basis.append({tuple(2 * x for x in e[i]): 2.0, e[i]: -1.0})
    for i, j in ((0, 1), (1, 2), (2, 0)):
        basis.append({tuple(x + y for x, y in zip(e[i], e[j])): 4.0})
    return np.array([[integrate(mul(p, q)) for q in basis] for p in basis])


def test_chebyshev_mass_bounds(oracle_lib, channel_coarse):
    """The Chebyshev mass solve (velocity method 3) relies on spec(D^-1 M) lying in
    [MASS_SPEC_LO, MASS_SPEC_HI] on every mesh: the element pair (M_e, diag M_e) has those extreme
    generalized eigenvalues (the same for every affine triangle), and the assembled spectrum
    lies inside them."""
    import scipy.linalg as sla
    O = oracle_lib
    Me = _p2_element_mass()
    assert abs(Me.sum() - 1.0) < 1e-14
    ev = sla.eigh(Me, np.diag(np.diag(Me)), eigvals_only=True)
    assert O.MASS_SPEC_LO <= ev.min() < O.MASS_SPEC_LO + 1e-5
    assert O.MASS_SPEC_HI - 1e-5 < ev.max() <= O.MASS_SPEC_HI
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, True)
    Md = ctx.M.to_scipy().toarray()
    d = np.diag(Md)
    g = sla.eigh(Md, np.diag(d), eigvals_only=True)
    assert O.MASS_SPEC_LO <= g.min() and g.max() <= O.MASS_SPEC_HI


def test_chebyshev_mass_solve(oracle_lib, channel_coarse):
    """The a priori count reaches the tolerance (true residual), and the solution matches a
    direct solve."""
    import scipy.sparse.linalg as spla
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, True)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(ctx.N)
    ref = spla.spsolve(ctx.M.to_scipy().tocsc(), b)
    for tol in (1e-6, 1e-10, 1e-13):
        k = O.cheb_iters(ctx.M, tol)
        x, st, rel = O.cheb_solve(ctx.M, b, k, tol)
        assert st == 0 and rel <= tol, (tol, k, rel)
        assert np.max(np.abs(x - ref)) <= 50 * tol * np.max(np.abs(ref))
    # fewer iterations than the count miss tight tolerances
    k = O.cheb_iters(ctx.M, 1e-10)
    _, st, rel = O.cheb_solve(ctx.M, b, k // 2, 1e-10)
    assert st == 3 and rel > 1e-10


def test_chebyshev_chorin_matches_pcg(oracle_lib, channel_coarse):
    """Chorin steps with the Chebyshev mass solve agree with the PCG ones at tight tolerances."""
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, True)
    a = O.Chorin(ctx, 1e-3, 1e-3, vel_method=1, vel_tol=1e-12, pres_tol=1e-12)
    b = O.Chorin(ctx, 1e-3, 1e-3, vel_method=3, vel_tol=1e-12, pres_tol=1e-12)
    for _ in range(5):
        a.step()
        st = b.step()
        assert st[0] == O.cheb_iters(ctx.M, 1e-12)
    ua, pa = a.state()
    ub, pb = b.state()
    assert np.max(np.abs(ua - ub)) <= 1e-9 * np.max(np.abs(ua))
    assert np.max(np.abs(pa - pb)) <= 1e-8 * np.max(np.abs(pa))


def test_projected_pressure_guess(oracle_lib, channel_coarse):
    """Pressure guess 2 (projection onto a Kp_int-orthonormal basis of earlier solutions, restarts
    from the solution and its last differences): the fields follow the previous-solution guess to
    the solver tolerance, and the solves get shorter once the basis holds a few vectors, across
    restarts of a small basis."""
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, True)
    runs = {}
    for guess, basis in ((0, 0), (2, 5), (2, 0)):
        ch = O.Chorin(ctx, 1e-3, 1e-3, vel_method=1, vel_tol=1e-12, pres_tol=1e-12, pres_guess=guess,
                      pres_basis=basis)
        its = [ch.step()[1] for _ in range(30)]
        runs[(guess, basis)] = (its, ch.state())
    its0, (u0, p0) = runs[(0, 0)]
    for key in ((2, 5), (2, 0)):
        its, (u, p) = runs[key]
        assert np.linalg.norm(u - u0) <= 1e-9 * np.linalg.norm(u0), key
        assert np.linalg.norm(p - p0) <= 1e-7 * np.linalg.norm(p0), key
        assert sum(its[10:]) < 0.9 * sum(its0[10:]), (key, its, its0)


def test_warm_chebyshev_mass_solves(oracle_lib, channel_coarse):
    """Mass-solve method 4 (Chebyshev from the previous step's solution, the count from the initial
    residual): the solves meet the tolerance, the fields follow the cold method 3, and the counts
    drop below the cold one once the flow settles."""
    O = oracle_lib
    m = O.Mesh(channel_coarse)
    ctx = O.Context(m, 1.2, True)
    cold = O.cheb_iters(ctx.M, 1e-10)
    a = O.Chorin(ctx, 1e-3, 1e-3, vel_method=3, vel_tol=1e-10, pres_tol=1e-12)
    b = O.Chorin(ctx, 1e-3, 1e-3, vel_method=4, vel_tol=1e-10, pres_tol=1e-12)
    its = []
    for _ in range(20):
        a.step()
        st = b.step()
        assert st[4] <= 1e-10 and st[5] <= 1e-10, st
        assert st[0] <= cold and st[2] <= cold
        its.append((st[0], st[2]))
    ua, pa = a.state()
    ub, pb = b.state()
    assert np.linalg.norm(ub - ua) <= 1e-8 * np.linalg.norm(ua)
    assert np.linalg.norm(pb - pa) <= 1e-7 * np.linalg.norm(pa)
    assert sum(t + f for t, f in its[10:]) < 0.9 * 2 * 10 * cold, its


# ------------------------------------------------------------ FP values: the reference's integrator
# The reference's element integrator (triangleIntegrator.cpp) and its CSR assembly (chorinCsr.cpp) run
# in FP32; the oracle and the product assemble in FP64 from the same float geometry.  Their values
# therefore agree to the FP32 rounding of the reference's own arithmetic: measured at most 4e-7 of the
# largest entry of each matrix on every mesh (1.0e-6 of the row's largest entry for the
# FastConvection matrix, whose rows mix entries of very different size).  The bounds below leave a
# factor 2.5 on that; a sign, transpose, node-order or quadrature error moves entries by O(1).
FP32_REL_GLOBAL = 1e-6   # |ours - ref| <= this * max |ref| over the matrix
FP32_REL_ROW = 2.5e-6    # |ours - ref| <= this * max |ref| over the row (+ 1e-7 max |ref| for empty rows)
ASSEMBLED = ("M", "K", "Kp", "D", "G", "I")


def _check_values(name, rs, cl, val, ref):
    assert np.array_equal(rs, ref.rowStart) and np.array_equal(cl, ref.col), name
    rv = ref.val.astype(np.float64)
    scale = np.abs(rv).max()
    d = np.abs(np.asarray(val, np.float64) - rv)
    assert d.max() <= FP32_REL_GLOBAL * scale, (name, d.max() / scale)
    rows = np.repeat(np.arange(ref.rows), np.diff(ref.rowStart))
    rmax = np.zeros(ref.rows)
    np.maximum.at(rmax, rows, np.abs(rv))
    assert np.all(d <= FP32_REL_ROW * rmax[rows] + 1e-7 * scale), name


@pytest.mark.parametrize("which", ["committed", "reference"])
def test_assembled_values_match_reference(oracle_lib, channel_coarse, which):
    """M, K, Kp, D, G from the reference's buildChorinCsrMatrices<float> and the FastConvection
    integration matrix I from its integrator, against the oracle's and the product's FP64 assembly."""
    import nsfemoptim_gb300 as G
    R = _reference()
    O = oracle_lib
    paths = [channel_coarse] if which == "committed" else _ref_meshes()
    if not paths:
        pytest.skip("reference meshes not present")
    for path in paths:
        h = R.ref_mesh_load(path.encode())
        assert h, R.ref_last_error()
        m = O.Mesh(path)
        ctx = O.Context(m, 1.2, True)
        pctx = G.build_chorin_context(G.load_gmsh(path), 1.2)
        for name in ASSEMBLED:
            ref = O.reference_assembled(R, h, name)
            a = getattr(ctx, name)
            _check_values(name, a.rowStart, a.col, a.val, ref)
            b = pctx.matrix(name)
            _check_values(name, b.rowStart, b.column, b.values, ref)
        R.ref_mesh_free(h)


def _local_fixture():
    return np.load(os.path.join(GOLDEN, "ref_local_channel_h0.025_s0.npz"))


def _check_local(ours, ref):
    for k, r in ref.items():
        o = ours[k]
        scale = np.abs(r).max()
        assert np.abs(o - r.astype(np.float64)).max() <= FP32_REL_GLOBAL * scale, k


def test_local_matrices_match_golden_reference(oracle_lib, channel_coarse):
    """The oracle's local element matrices (mass, stiffness, P1 stiffness, divergence, gradient and
    the twelve unit-velocity self-convection matrices) against the reference integrator's, stored
    for a seeded sample of elements of the committed mesh (tests/golden/make_golden.py).  Runs
    without the reference tree."""
    O = oracle_lib
    fx = _local_fixture()
    m = O.Mesh(channel_coarse)
    for i, e in enumerate(fx["elements"]):
        _check_local(m.local_matrices(int(e)), {k: fx[k][i] for k, _ in O.Mesh.LOCAL_SHAPES})


def test_local_matrices_match_live_reference(oracle_lib, channel_coarse):
    """The same on every element of the committed mesh and of the shipped h = 0.025 mesh, against
    the reference integrator compiled here."""
    R = _reference()
    O = oracle_lib
    paths = [channel_coarse] + [p for p in _ref_meshes() if p.endswith("h_0.025.msh")]
    for path in paths:
        h = R.ref_mesh_load(path.encode())
        m = O.Mesh(path)
        for e in range(m.num_tri):
            _check_local(m.local_matrices(e), O.reference_local_matrices(R, h, e))
        R.ref_mesh_free(h)

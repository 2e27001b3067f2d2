"""Which parts of a preconditioned CG may run in FP32 without delaying it on an ill-conditioned
system: the evidence behind the mixed solve of the cooperative-grid path (one CG with the FP64
recurrence and A p under an FP32 SGS preconditioner).

System: P1 Laplacian of a jittered 128 x 128-node unit square (seed 0, jitter 0.2 h), pinned at
node 0, right-hand side N(0, 1) (seed 0) projected to zero mean; multicolor SGS in the smallest-last
greedy colouring of the oracle; CG to 1e-10 on the FP64 residual.  numpy/scipy emulation of each
arithmetic split (float32 arrays for the FP32 parts), run on the CPU:

  FP64 everything                                  402 iterations
  FP64 recurrence and A p, FP32 SGS preconditioner 402
  FP32 everything, FP64 residual replacement       558
  FP32 values of A in A p, FP64 arithmetic         559

(1,585 / 1,585 / 4,603 / 2,394 at 512 x 512 nodes: the delay grows with the condition number.)
"""

import numpy as np
import pytest


@pytest.fixture(scope="module")
def system(oracle_lib):
    import scipy.sparse as sp

    from nsfemoptim_gb300 import meshgen
    O = oracle_lib
    mesh = meshgen.jittered_square(128, seed=0, jitter=0.2)
    rs, ci, val = meshgen.p1_stiffness(mesh.nodes, mesh.triangles)
    full = sp.csr_matrix((val, ci, rs))
    full.sort_indices()
    A = full[1:, 1:].tocsr()
    A.sort_indices()
    n = A.shape[0]
    b = np.random.default_rng(0).standard_normal(n + 1)
    b = (b - b.mean())[1:]
    oc = O.Csr(n, n, A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data)
    perm, part, _ = O.coloring(oc)
    P = sp.csr_matrix((np.ones(n), (np.arange(n), np.asarray(perm))), shape=(n, n))
    Ap = (P @ A @ P.T).tocsr()
    Ap.sort_indices()
    return Ap, P @ b, np.asarray(part)


def _sgs_parts(A, part, dt):
    C = len(part) - 1
    M = A.astype(dt)
    L = [M[part[c]:part[c + 1], :part[c]].tocsr() for c in range(C)]
    U = [M[part[c]:part[c + 1], part[c + 1]:].tocsr() for c in range(C)]
    return L, U, (1.0 / M.diagonal()).astype(dt)


def _sgs(r, L, U, invD, part):
    """Multicolor symmetric Gauss-Seidel from z = 0: forward over the colours, backward over all but
    the last (the order of the device sweeps)."""
    C = len(part) - 1
    y = np.zeros_like(r)
    for c in range(C):
        s, e = part[c], part[c + 1]
        y[s:e] = invD[s:e] * (r[s:e] - (L[c] @ y[:s] if s > 0 else 0))
    for c in range(C - 2, -1, -1):
        s, e = part[c], part[c + 1]
        y[s:e] = y[s:e] - invD[s:e] * (U[c] @ y[e:])
    return y


def _cg(A, b, part, op32=False, pre32=False, vec32=False, tol=1e-10, delta=0.1):
    """PCG with FP64 residual replacement (r = b - A x in FP64 whenever the recurrence's |r| has
    dropped by delta): op32 applies A with FP32-rounded values, pre32 runs the preconditioner in
    FP32, vec32 keeps r, p, q and the increment of x in FP32 (with A p rounded to FP32)."""
    f = np.float32 if vec32 else np.float64
    Aop = A.astype(np.float32).astype(np.float64) if op32 else A
    pd = np.float32 if pre32 else np.float64
    L, U, invD = _sgs_parts(A, part, pd)

    def prec(v):
        return _sgs(v.astype(pd), L, U, invD, part).astype(f)

    bn = np.linalg.norm(b)
    x = np.zeros(len(b))
    r = b.astype(f)
    dx = np.zeros(len(b), f)
    z = prec(r)
    p = z.copy()
    rho = float(r.astype(np.float64) @ z)
    rmax = float(r.astype(np.float64) @ r)
    for k in range(1, 20000):
        q = (Aop @ p.astype(np.float64)).astype(f)
        a = rho / float(p.astype(np.float64) @ q)
        dx += f(a) * p
        r -= f(a) * q
        rr = float(r.astype(np.float64) @ r)
        if rr <= delta * delta * rmax or rr <= (tol * bn) ** 2:
            x += dx.astype(np.float64)
            dx[:] = 0
            r64 = b - A @ x
            if np.linalg.norm(r64) <= tol * bn:
                return k
            r = r64.astype(f)
            rmax = float(r64 @ r64)
        z = prec(r)
        rn = float(r.astype(np.float64) @ z)
        p = z + f(rn / rho) * p
        rho = rn
    return -1


def test_fp32_preconditioner_alone_keeps_the_fp64_iterations(system):
    A, b, part = system
    k64 = _cg(A, b, part)
    kpre = _cg(A, b, part, pre32=True)
    kall = _cg(A, b, part, op32=True, pre32=True, vec32=True)
    kop = _cg(A, b, part, op32=True)
    assert k64 > 300
    assert abs(kpre - k64) <= 2, (k64, kpre)
    assert kall >= 1.25 * k64, (k64, kall)
    assert kop >= 1.25 * k64, (k64, kop)

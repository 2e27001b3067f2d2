"""Pure-Neumann Poisson with one pin and the zero-mean correction on the device (nsf_neumann_*),
through the C ABI, against the FP64 oracle solving the same pinned system.

System: the P1 Laplacian of the committed jittered 33 x 33 unit square (1,089 nodes, no Dirichlet
node: its null space is the constants), pin at node 0, right-hand side N(0, 1) from seed 4 (not of
zero mean: the device projects it).  The oracle solves the pinned system with the same PCG-SGS to
1e-13 relative and the test shifts its solution to zero mean in numpy.

Bounds: FP64 and mixed solves to 1e-10 relative residual of the pinned system; the solution within
5e-9 (relative L2) of the oracle's, about 10x the largest error measured on a GB300 (FP64 2.0e-11,
mixed 4.6e-10); the mean of the solution below 1e-13 of its largest entry; the full singular
system's residual K x - (b - mean(b)) below 1e-9 of the projected right-hand side.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def laplacian(square_small, oracle_lib):
    import scipy.sparse as sp

    from nsfemoptim_gb300 import meshgen
    from nsfemoptim_gb300.api import HostCsr
    O = oracle_lib
    m = O.Mesh(square_small)
    rs, ci, val = meshgen.p1_stiffness(m.corner_xy.astype(np.float64), m.tri)
    K = sp.csr_matrix((val, ci, rs))
    K.sort_indices()
    n = K.shape[0]
    host = HostCsr(n, n, K.indptr.astype(np.int32), K.indices.astype(np.int32), K.data.copy())
    b = np.random.default_rng(4).standard_normal(n)
    bp = b - b.mean()
    Kr = K[1:, 1:].tocsr()
    Kr.sort_indices()
    oc = O.Csr(n - 1, n - 1, Kr.indptr.astype(np.int32), Kr.indices.astype(np.int32), Kr.data.copy())
    xr, st, it, rr = O.pcg(oc, O.coloring(oc), bp[1:], np.zeros(n - 1), 20000, 1e-13)
    assert st == 0
    xo = np.concatenate([[0.0], xr])
    xo -= xo.mean()
    return K, host, b, bp, xo


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_neumann_pin_zero_mean_matches_oracle(torch_cuda, laplacian, precision):
    import nsfemoptim_gb300 as G
    t = torch_cuda
    K, host, b, bp, xo = laplacian
    prec = G.NSF_PREC_F64 if precision == "f64" else G.NSF_PREC_MIXED
    s = G.NeumannSolver(host, pin=0, precision=prec, max_iters=5000, target=1e-10)
    bd = t.tensor(b, device="cuda")
    for guess in (np.zeros(len(b)), np.random.default_rng(5).standard_normal(len(b))):
        xd = t.tensor(guess, device="cuda")
        s.solve(bd, xd)
        x = xd.cpu().numpy()
        st = s.stats()
        err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
        print(f"neumann {precision}: rel err {err:.3e} iters {st['iters']} rel {st['rel']:.3e} "
              f"mean {x.mean():.3e}")
        assert st["rel"] <= 1e-10
        assert err <= 5e-9
        assert abs(x.mean()) <= 1e-13 * np.abs(x).max()
        assert np.linalg.norm(K @ x - bp) <= 1e-9 * np.linalg.norm(bp)


def test_neumann_rejects_bad_pin(torch_cuda, laplacian):
    import nsfemoptim_gb300 as G
    K, host, b, bp, xo = laplacian
    with pytest.raises(G.NsfError):
        G.NeumannSolver(host, pin=host.rows)


@pytest.fixture(scope="module")
def laplacian_256():
    """P1 Laplacian of a jittered 256 x 256-node unit square (seed 0), the config-3 family at 1/16 of
    its size: condition number ~1e5 after pinning."""
    import scipy.sparse as sp

    from nsfemoptim_gb300 import meshgen
    from nsfemoptim_gb300.api import HostCsr
    mesh = meshgen.jittered_square(256, seed=0, jitter=0.2)
    rs, ci, val = meshgen.p1_stiffness(mesh.nodes, mesh.triangles)
    K = sp.csr_matrix((val, ci, rs))
    K.sort_indices()
    n = K.shape[0]
    host = HostCsr(n, n, K.indptr.astype(np.int32), K.indices.astype(np.int32), K.data.copy())
    b = np.random.default_rng(0).standard_normal(n)
    return K, host, b, b - b.mean()


def test_mixed_grid_solve_keeps_fp64_iterations(torch_cuda, laplacian_256, monkeypatch):
    """On the cooperative-grid path a mixed solve is one CG with the FP64 recurrence and A p under
    the FP32 SGS preconditioner: it needs the FP64 solve's iterations (within 2% + 2) to the same
    1e-10 on the FP64 residual, where restarted FP32 refinement passes (NSF_MIXED_FORM=refine) need
    far more.  Both grid row layouts (4 lanes per row, one thread per row) give the same counts."""
    import nsfemoptim_gb300 as G
    t = torch_cuda
    K, host, b, bp = laplacian_256
    monkeypatch.setenv("NSF_PCG_PATH", "grid")
    bd = t.tensor(b, device="cuda")
    its = {}
    for lanes in ("4", "1"):
        monkeypatch.setenv("NSF_GRID_LANES", lanes)
        for form in ("auto", "refine"):
            monkeypatch.setenv("NSF_MIXED_FORM", form)
            for name, prec in (("f64", G.NSF_PREC_F64), ("mixed", G.NSF_PREC_MIXED)):
                if name == "f64" and form == "refine":
                    continue
                s = G.NeumannSolver(host, pin=0, precision=prec, max_iters=20000, target=1e-10)
                xd = t.zeros(len(b), dtype=t.float64, device="cuda")
                s.solve(bd, xd)
                x = xd.cpu().numpy()
                st = s.stats()
                assert st["rel"] <= 1e-10, (lanes, form, name, st)
                assert np.linalg.norm(K @ x - bp) <= 1e-9 * np.linalg.norm(bp)
                its[(lanes, form, name)] = st["iters"]
        f64, mixed = its[(lanes, "auto", "f64")], its[(lanes, "auto", "mixed")]
        print(f"lanes {lanes}: FP64 {f64}, mixed {mixed}, refine {its[(lanes, 'refine', 'mixed')]}")
        assert mixed <= 1.02 * f64 + 2, its
        assert its[(lanes, "refine", "mixed")] >= 1.2 * f64, its
    assert abs(its[("4", "auto", "f64")] - its[("1", "auto", "f64")]) <= 2

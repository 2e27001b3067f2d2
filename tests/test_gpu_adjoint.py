"""GPU discrete adjoint (nsf_adjoint_*) against the FP64 CPU adjoint of the oracle and against FP64
central finite differences of the GPU forward run (torch.autograd.gradcheck through the harness of
nsfemoptim_gb300.gradcheck).  No reference counterpart exists; these are the pins.

Tolerances:
  GPU vs oracle adjoint (same discrete step, solves to 1e-13 / 1e-14):  J rel 1e-11,
      dJ/dnu rel 1e-8, dJ/d dirVx and dJ/du0 normwise rel 1e-8
  checkpoint interval 0 / 3 / 5 and binomial checkpointing with 1 / 2 / 3 / 8 stored states:
      bit-identical results (the recomputation replays the same kernels)
  adjoint vs central FD (eps = 1e-6):  rel 1e-6 per component (gradcheck rtol), atol 1e-6 x max|g|
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NU, TAU, PEAK = 1e-3, 5e-4, 4.0  # U_max = PEAK / 4 = 1.0


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def adj_setup(torch_cuda, channel_coarse, oracle_lib):
    import nsfemoptim_gb300 as G
    O = oracle_lib
    mesh = G.load_gmsh(channel_coarse)
    ctx = G.build_chorin_context(mesh, PEAK)
    om = O.Mesh(channel_coarse)
    oc = O.Context(om, PEAK, True)
    return G, O, mesh, ctx, om, oc


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def _stepper(G, ctx, tol=1e-13, precision=None, vel_method=1):
    prec = G.NSF_PREC_F64 if precision in (None, "f64") else G.NSF_PREC_F64_MIXEDSOLVE
    return G.ChorinStepper(ctx, NU, TAU, precision=prec, vel_method=vel_method, vel_max_iters=20000, vel_tol=tol,
                           pres_max_iters=20000, pres_tol=tol, use_graph=True, max_outer=6, inner_tol=1e-5)


def _start(rng, n_nodes):
    u0 = np.zeros(2 * n_nodes)
    u0[:n_nodes] = 0.3 * rng.random(n_nodes)
    u0[n_nodes:] = 0.05 * rng.standard_normal(n_nodes)
    return u0


@pytest.mark.parametrize("precision,vel_method", [("f64", 1), ("mixedsolve", 1), ("f64", 2), ("mixedsolve", 2),
                                                  ("f64", 3), ("mixedsolve", 3)])
def test_adjoint_matches_oracle_adjoint(adj_setup, precision, vel_method):
    """Drag and lift weights on every step, a random initial velocity and perturbed inflow values.
    mixedsolve: FP64 operators with FP32-inner solves refined to the same FP64 tolerance, in the
    forward step and in the adjoint solves.  vel_method 2: Jacobi-preconditioned mass solves, 3:
    Chebyshev-Jacobi mass solves (the discrete step is the same; only the solver differs, within
    the tolerance)."""
    G, O, mesh, ctx, om, oc = adj_setup
    rng = np.random.default_rng(11)
    n = 12
    wd, wl = rng.random(n), rng.standard_normal(n)
    u0 = _start(rng, ctx.N)
    dv = ctx.dir_vx + 0.01 * rng.standard_normal(len(ctx.dir_vx)) * (ctx.dir_vx != 0)
    st = _stepper(G, ctx, precision=precision, vel_method=vel_method)
    f = G.Forces(mesh, st)
    adj = G.Adjoint(st, f, checkpoint_interval=0, tol=1e-13)
    st.set_state(u0, np.zeros(ctx.P))
    st.set_dirichlet(dv)
    J, gnu, gdir, gu = adj.run(n, wd, wl)
    s = adj.stats()
    # mixed solves may stop at the FP64 residual floor just above 1e-13 (status 3, reported only)
    ok = (0,) if precision == "f64" else (0, 3)
    assert s["forward_status"] in ok and s["adjoint_status"] in ok
    assert s["reverse_steps"] == n and s["recomputed_steps"] == 0
    Jo, gnuo, gdiro, guo = O.adjoint_run(oc, om, NU, TAU, n, wd, wl, dir_vx=dv, u0=u0, vel_tol=1e-14,
                                         pres_tol=1e-14, solve_tol=1e-14)
    assert abs(J - Jo) <= 1e-11 * abs(Jo)
    assert abs(gnu - gnuo) <= 1e-8 * abs(gnuo)
    assert _rel(gdir, gdiro) <= 1e-8
    assert _rel(gu, guo) <= 1e-8
    assert np.all(gu[ctx.dir_ids] == 0) and np.all(gu[ctx.N + ctx.dir_ids] == 0)
    # the stepper ends in the state after the forward run
    ue, _ = st.state()
    ch = O.Chorin(oc, NU, TAU, vel_method=1, vel_max_iters=20000, vel_tol=1e-14, pres_max_iters=20000,
                  pres_tol=1e-14)
    ch.set_state(u0, np.zeros(ctx.P))
    ch.set_dirichlet(dv)
    for _ in range(n):
        ch.step()
    assert _rel(ue, ch.state()[0]) <= 1e-9


def test_mixedsolve_step_matches_fp64_step(adj_setup):
    """NSF_PREC_F64_MIXEDSOLVE keeps the FP64 step: its states follow the FP64 stepper's to the
    solver tolerance (1e-12 here) over 6 steps; every solve reports convergence."""
    G, O, mesh, ctx, om, oc = adj_setup
    rng = np.random.default_rng(14)
    u0 = _start(rng, ctx.N)
    a, b = _stepper(G, ctx, 1e-12), _stepper(G, ctx, 1e-12, "mixedsolve")
    for st in (a, b):
        st.set_state(u0, np.zeros(ctx.P))
        st.set_dirichlet(ctx.dir_vx)
    for _ in range(6):
        a.step(1)
        b.step(1)
        assert b.stats()["status"] == 0
        assert max(b.stats()["tent_rel"], b.stats()["pres_rel"], b.stats()["final_rel"]) <= 1e-12
    ua, pa = a.state()
    ub, pb = b.state()
    assert _rel(ub, ua) <= 1e-10
    assert _rel(pb, pa) <= 1e-8


def test_checkpointing_is_exact(adj_setup):
    """Recomputing segments from checkpoints gives the same bits as keeping every state."""
    G, O, mesh, ctx, om, oc = adj_setup
    rng = np.random.default_rng(12)
    n = 11
    wd = np.zeros(n)
    wd[4:9] = rng.random(5)  # trailing unweighted steps: the reverse sweep starts at step 8
    u0 = _start(rng, ctx.N)
    st = _stepper(G, ctx)
    f = G.Forces(mesh, st)
    out = {}
    for c in (0, 3, 5):
        adj = G.Adjoint(st, f, checkpoint_interval=c)
        st.set_state(u0, np.zeros(ctx.P))
        st.set_dirichlet(ctx.dir_vx)
        out[c] = adj.run(n, wd)
        s = adj.stats()
        assert s["reverse_steps"] == 9
        if c:
            segs = -(-9 // c)
            assert s["recomputed_steps"] == 9 - segs
    for c in (3, 5):
        assert out[c][0] == out[0][0] and out[c][1] == out[0][1]
        assert np.array_equal(out[c][2], out[0][2]) and np.array_equal(out[c][3], out[0][3])


def _binomial_recomputations(k, s):
    """Fewest recomputed steps to reverse k steps with s stored states besides the first:
    R(1, s) = 0, R(k, 0) = k (k - 1) / 2, R(k, s) = min_m m + R(k - m, s - 1) + R(m, s)."""
    R = [[0] * (s + 1) for _ in range(k + 1)]
    for kk in range(1, k + 1):
        R[kk][0] = kk * (kk - 1) // 2
    for ss in range(1, s + 1):
        for kk in range(2, k + 1):
            R[kk][ss] = min(m + R[kk - m][ss - 1] + R[m][ss] for m in range(1, kk))
    return R[k][s]


def test_binomial_checkpointing_is_exact(adj_setup):
    """Binomial checkpointing (snapshots > 0) gives the same bits as keeping every state, with the
    fewest recomputed steps for its memory (the binomial recursion's optimum) and (s + 1) stored
    states."""
    G, O, mesh, ctx, om, oc = adj_setup
    rng = np.random.default_rng(13)
    n = 11
    wd = np.zeros(n)
    wd[4:9] = rng.random(5)  # the reverse sweep covers steps 0..8
    u0 = _start(rng, ctx.N)
    st = _stepper(G, ctx)
    f = G.Forces(mesh, st)

    def run(**kw):
        adj = G.Adjoint(st, f, **kw)
        st.set_state(u0, np.zeros(ctx.P))
        st.set_dirichlet(ctx.dir_vx)
        return adj.run(n, wd), adj.stats()

    ref, _ = run(checkpoint_interval=0)
    for snaps in (1, 2, 3, 8):
        out, s = run(snapshots=snaps)
        assert s["reverse_steps"] == 9
        assert s["recomputed_steps"] == _binomial_recomputations(9, snaps), (snaps, s["recomputed_steps"])
        assert out[0] == ref[0] and out[1] == ref[1]
        assert np.array_equal(out[2], ref[2]) and np.array_equal(out[3], ref[3])


def test_set_nu_changes_the_forward_run(adj_setup):
    """The viscosity setter reaches the captured step: J(nu +- eps) differ by about 2 eps dJ/dnu."""
    G, O, mesh, ctx, om, oc = adj_setup
    from nsfemoptim_gb300 import gradcheck as GC
    n = 8
    prob = GC.DragProblem(mesh, ctx, PEAK, NU, TAU, n, np.full(n, 1.0 / n), n_coef=2, checkpoint_interval=0)
    th = np.zeros(2)
    J, gnu, _, _ = prob.gradient(NU, th)
    eps = 1e-6
    fd = (prob.value(NU + eps, th) - prob.value(NU - eps, th)) / (2 * eps)
    assert abs(fd - gnu) <= 1e-5 * abs(gnu), (fd, gnu)
    assert abs(prob.value(NU, th) - J) <= 1e-13 * abs(J)


def test_adjoint_gradcheck_central_differences(adj_setup, torch_cuda):
    """torch.autograd.gradcheck of the harness: the adjoint's d/dnu and d/dtheta (4 inflow sine
    coefficients) against FP64 central differences with eps = 1e-6 of the GPU forward run."""
    torch = torch_cuda
    G, O, mesh, ctx, om, oc = adj_setup
    from nsfemoptim_gb300 import gradcheck as GC
    n = 16
    w = np.zeros(n)
    w[n // 2:] = 1.0 / (n - n // 2)
    prob = GC.DragProblem(mesh, ctx, PEAK, NU, TAU, n, w, n_coef=4, tol=1e-13, checkpoint_interval=5)
    rng = np.random.default_rng(13)
    nu = torch.tensor([NU], dtype=torch.float64, requires_grad=True)
    theta = torch.tensor(0.01 * rng.standard_normal(4), dtype=torch.float64, requires_grad=True)
    J, gnu, gth, _ = prob.gradient(NU, theta.detach().numpy())
    assert abs(prob.value(NU, theta.detach().numpy()) - J) <= 1e-13 * abs(J)
    atol = 1e-6 * max(abs(gnu), float(np.abs(gth).max()))
    assert torch.autograd.gradcheck(lambda a, b: GC.drag(prob, a, b), (nu, theta), eps=1e-6, atol=atol, rtol=1e-6)


def test_adjoint_rejects_mixed_stepper(adj_setup):
    G, O, mesh, ctx, om, oc = adj_setup
    st = G.ChorinStepper(ctx, NU, TAU, precision=G.NSF_PREC_MIXED, vel_method=1)
    f = G.Forces(mesh, st)
    with pytest.raises(G.NsfError):
        G.Adjoint(st, f)

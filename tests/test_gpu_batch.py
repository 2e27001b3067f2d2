"""Batched instances (nsf_batch_*) against separate steppers, through the C ABI.

Three instances on the committed h = 0.025 channel mesh with their own viscosities (1e-3, 2e-3,
5e-4) and inflow values (the context's scaled by 1.0, 0.7, 1.3), tau = 1e-3, mixed precision,
Chebyshev mass solves to 1e-10, pressure to 1e-10, pressure guess 0, 1 and 2 (a 4-vector projection
basis, so 5 steps pass through a restart): after 5 steps every
instance's state equals, bit for bit, the state of a ChorinStepper with the same options (the batched
kernels run the single stepper's arithmetic, instance by instance).  set_state / state round trip
and the per-instance statistics are checked too.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NUS = [1e-3, 2e-3, 5e-4]
SCALES = [1.0, 0.7, 1.3]


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def ctx(torch_cuda, channel_coarse):
    import nsfemoptim_gb300 as G
    return G, G.build_chorin_context(G.load_gmsh(channel_coarse), 1.2)


@pytest.mark.parametrize("coarse", ["0", "1"])
@pytest.mark.parametrize("guess", [0, 1, 2])
def test_batch_equals_separate_steppers(ctx, guess, coarse, monkeypatch):
    """coarse: the pressure preconditioner, SGS alone (Eisenstat's kernel) or SGS plus the coarse
    correction (the classical kernel), the same in the batch and in the steppers."""
    G, c = ctx
    monkeypatch.setenv("NSF_BATCH_CLUSTER", "16")  # the cluster size of a single solve: the same reduction order
    monkeypatch.setenv("NSF_PRES_COARSE", coarse)
    dir_vx = np.stack([c.dir_vx * s for s in SCALES])
    b = G.Batch(c, NUS, 1e-3, dir_vx=dir_vx, vel_tol=1e-10, pres_tol=1e-10, pressure_guess=guess, pressure_basis=4)
    b.step(5)
    assert b.kernels_per_step() > 0
    for q, (nu, sc) in enumerate(zip(NUS, SCALES)):
        st = G.ChorinStepper(c, nu, 1e-3, precision=G.NSF_PREC_MIXED, vel_method=3, vel_max_iters=500, vel_tol=1e-10,
                             pres_max_iters=5000, pres_tol=1e-10, use_graph=True, max_outer=4, inner_tol=1e-5,
                             pressure_guess=guess, pressure_basis=4)
        st.set_dirichlet(dir_vx[q])
        st.step(5)
        u, p = st.state()
        ub, pb = b.state(q)
        assert np.array_equal(u, ub) and np.array_equal(p, pb), (q, np.abs(u - ub).max(), np.abs(p - pb).max())
        s = b.stats(q)
        assert s["status"] == 0 and s["pres_rel"] <= 1e-10
        assert s["pres_iters"] == st.stats()["pres_iters"]


def test_batch_state_roundtrip(ctx):
    G, c = ctx
    b = G.Batch(c, NUS, 1e-3, vel_tol=1e-10, pres_tol=1e-10)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(2 * c.N)
    p = np.zeros(c.P)
    p[c.int_p] = rng.standard_normal(len(c.int_p))
    b.set_state(1, u, p)
    u2, p2 = b.state(1)
    assert np.array_equal(u, u2) and np.array_equal(p, p2)
    with pytest.raises(G.NsfError):
        b.state(3)


def test_batch_small_clusters_follow_steppers(ctx, monkeypatch):
    """With the batch's own cluster size (smaller clusters, so that more instances' pressure solves
    run at once) only the summation order of the pressure CG's dot products changes: the states
    follow the separate steppers to the solver tolerance: 10x the measured relative differences
    (u 2.6e-12, p 2.1e-9 with pressure solves to 1e-10).  The steppers use the batch's single-level
    pressure preconditioner."""
    G, c = ctx
    monkeypatch.setenv("NSF_PRES_COARSE", "0")
    dir_vx = np.stack([c.dir_vx * s for s in SCALES])
    b = G.Batch(c, NUS, 1e-3, dir_vx=dir_vx, vel_tol=1e-10, pres_tol=1e-10, pressure_guess=2, pressure_basis=4)
    b.step(5)
    for q, nu in enumerate(NUS):
        st = G.ChorinStepper(c, nu, 1e-3, precision=G.NSF_PREC_MIXED, vel_method=3, vel_max_iters=500, vel_tol=1e-10,
                             pres_max_iters=5000, pres_tol=1e-10, use_graph=True, max_outer=4, inner_tol=1e-5,
                             pressure_guess=2, pressure_basis=4)
        st.set_dirichlet(dir_vx[q])
        st.step(5)
        u, p = st.state()
        ub, pb = b.state(q)
        eu = np.linalg.norm(u - ub) / np.linalg.norm(u)
        ep = np.linalg.norm(p - pb) / np.linalg.norm(p)
        print(f"instance {q}: u {eu:.3e} p {ep:.3e}")
        assert eu <= 3e-11 and ep <= 2e-8


def test_pack_of_batches_equals_batches_alone(ctx, channel_h01):
    """A pack of batches (nsf_pack_create_batches: one graph whose branches are the batched steps,
    here a batch on the h = 0.025 mesh and one on the h = 0.01 mesh) leaves every instance's state bit
    for bit where the same batches stepped on their own leave it: the branches share nothing."""
    G, c = ctx
    fine = G.build_chorin_context(G.load_gmsh(channel_h01), 1.2)
    dir_vx = np.stack([c.dir_vx * s for s in SCALES])

    def make():
        return [G.Batch(c, NUS, 1e-3, dir_vx=dir_vx, vel_tol=1e-10, pres_tol=1e-10, pressure_guess=2,
                        pressure_basis=4),
                G.Batch(fine, NUS[:2], 5e-4, vel_tol=1e-10, pres_tol=1e-10, pressure_guess=1)]

    alone = make()
    for b in alone:
        b.step(4)
    packed = make()
    pack = G.Pack(packed)
    assert pack.kernels_per_step() == sum(b.kernels_per_step() for b in alone)
    pack.step(4)
    import torch
    torch.cuda.synchronize()
    for a, b in zip(alone, packed):
        for q in range(a.B):
            ua, pa = a.state(q)
            ub, pb = b.state(q)
            assert np.array_equal(ua, ub) and np.array_equal(pa, pb), q
            assert b.stats(q)["status"] == 0


def test_batch_mass_solve_groups_do_not_change_results(ctx, monkeypatch):
    """The instances of the batched mass solves run in L2-sized groups (NSF_BATCH_CHEB_GROUP: a
    size, or `tune` to time every power of two and keep the fastest); per instance the arithmetic
    is the same whatever the grouping, so the states are bitwise those of the ungrouped batch."""
    G, c = ctx
    dir_vx = np.stack([c.dir_vx * s for s in SCALES])
    out = {}
    for group in ("3", "1", "2", "tune"):
        monkeypatch.setenv("NSF_BATCH_CHEB_GROUP", group)
        b = G.Batch(c, NUS, 1e-3, dir_vx=dir_vx, vel_tol=1e-10, pres_tol=1e-10, pressure_guess=2, pressure_basis=4)
        b.step(3)
        out[group] = [b.state(q) for q in range(3)]
    for group in ("1", "2", "tune"):
        for q in range(3):
            assert np.array_equal(out[group][q][0], out["3"][q][0]), (group, q)
            assert np.array_equal(out[group][q][1], out["3"][q][1]), (group, q)

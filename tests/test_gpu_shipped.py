"""GPU parity at full size, through the C ABI, against the FP64 C oracle running the same options.

Meshes:
  * the reference's shipped h_0.01 channel mesh (cpp/assets/h_0.01.msh, 20,970 triangles), read from
    the reference tree or from the copy that the reference harness build leaves in oracle/_ref/assets;
    skipped where neither exists;
  * the bench configuration: the seeded synthetic h = 0.005 channel (82,743 triangles), U_max = 1.5
    (peak inflow 6.0), nu = 1e-3, tau = 1e-4, Chebyshev mass solves, the projected pressure guess,
    pressure to 1e-8 relative.

Bounds (relative L2 over the whole field; each is about 10x the largest value measured on a GB300):
  FP64 stepper vs FP64 oracle, 5 steps            u, p <= 5e-12 (measured: u 5.8e-14, p 3.5e-13)
  mixed stepper vs FP64 oracle, 5 steps           u, p <= 4e-6  (measured: u 2.7e-7, p 3.9e-7)
  mixed stepper vs FP64 oracle, 100 steps, h_0.01 u, p <= 4e-7  (measured: u 2.4e-8, p 3.7e-8)
"""

import os

import numpy as np
import pytest

from conftest import shipped_mesh_path

pytestmark = pytest.mark.gpu

F64_BOUND = 5e-12
MIXED_5_BOUND = 4e-6
MIXED_100_BOUND = 4e-7


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def shipped_h01(torch_cuda, oracle_lib):
    path = shipped_mesh_path("h_0.01.msh")
    if path is None:
        pytest.skip("the reference's shipped h_0.01 mesh is not present")
    import nsfemoptim_gb300 as G
    O = oracle_lib
    peak = 4.0  # U_max = 1.0
    ctx = G.build_chorin_context(G.load_gmsh(path), peak)
    oc = O.Context(O.Mesh(path), peak, True)
    return G, O, ctx, oc


@pytest.fixture(scope="module")
def bench_h005(torch_cuda, oracle_lib, mesh_dir):
    import nsfemoptim_gb300 as G
    from nsfemoptim_gb300 import meshgen
    O = oracle_lib
    path = os.path.join(mesh_dir, "channel_h0.005_s0.msh")
    if not os.path.exists(path):
        meshgen.write_gmsh41(path, meshgen.dfg_channel(0.005, seed=0))
    peak = 6.0  # U_max = 1.5
    ctx = G.build_chorin_context(G.load_gmsh(path), peak)
    oc = O.Context(O.Mesh(path), peak, True)
    return G, O, ctx, oc


# (nu, tau, pressure tolerance, velocity tolerance) of each configuration
H01 = (1e-3, 5e-4, 1e-10, 1e-10)
H005 = (1e-3, 1e-4, 1e-8, 1e-8)


def _gpu(G, ctx, cfg, precision, vel_method=3, guess=2):
    nu, tau, ptol, vtol = cfg
    prec = {"f64": G.NSF_PREC_F64, "mixed": G.NSF_PREC_MIXED}[precision]
    return G.ChorinStepper(ctx, nu, tau, precision=prec, vel_method=vel_method, vel_max_iters=500, vel_tol=vtol,
                           pres_max_iters=5000, pres_tol=ptol, use_graph=True, max_outer=4, inner_tol=1e-5,
                           pressure_guess=guess)


def _oracle(O, oc, cfg, vel_method=3, guess=2):
    nu, tau, ptol, vtol = cfg
    return O.Chorin(oc, nu, tau, vel_method=vel_method, vel_max_iters=500, vel_tol=vtol, pres_max_iters=5000,
                    pres_tol=ptol, pres_guess=guess)


def _compare(st, ch, steps):
    st.step(steps)
    for _ in range(steps):
        ch.step()
    u, p = st.state()
    uo, po = ch.state()
    return _rel(u, uo), _rel(p, po)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
@pytest.mark.parametrize("case", ["shipped_h0.01", "bench_h0.005"])
def test_chorin_full_size_matches_oracle(request, precision, case):
    """5 steps from rest of the FP64 and the mixed stepper (Chebyshev mass solves, projected pressure
    guess, graph-captured) against the FP64 oracle with the same options."""
    G, O, ctx, oc = request.getfixturevalue("shipped_h01" if case == "shipped_h0.01" else "bench_h005")
    cfg = H01 if case == "shipped_h0.01" else H005
    st = _gpu(G, ctx, cfg, precision)
    eu, ep = _compare(st, _oracle(O, oc, cfg), 5)
    print(f"{case} {precision} 5 steps: u {eu:.3e} p {ep:.3e} stats {st.stats()}")
    bound = F64_BOUND if precision == "f64" else MIXED_5_BOUND
    assert st.stats()["status"] == 0
    assert eu <= bound and ep <= bound, (eu, ep)


def test_chorin_mixed_100_steps_shipped_h01(shipped_h01):
    """The mixed stepper over 100 steps on the shipped h_0.01 mesh against the FP64 oracle: the
    FP32 inner solves and the double-float products must not drift beyond the solver tolerance."""
    G, O, ctx, oc = shipped_h01
    st = _gpu(G, ctx, H01, "mixed")
    eu, ep = _compare(st, _oracle(O, oc, H01), 100)
    print(f"shipped_h0.01 mixed 100 steps: u {eu:.3e} p {ep:.3e} stats {st.stats()}")
    assert st.stats()["status"] == 0
    assert eu <= MIXED_100_BOUND and ep <= MIXED_100_BOUND, (eu, ep)

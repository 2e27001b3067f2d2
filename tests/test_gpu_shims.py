"""The reference-shaped time-step loop (tests/shims/chorin_loop.cpp: solveNsChorinCuda's loop written
against the cu:: shims of include/cu_gb300_shims.hpp, FP32 vectors and operators as the reference's)
against this library's own stepper (nsf_chorin_step, FP64), 3 steps on the committed h = 0.025
channel mesh (peak inflow 1.2, nu = 1e-3, tau = 1e-3; velocity and pressure CG with the multicolor
SGS preconditioner to 1e-8 relative, pressure warm-started from the previous solution).

The loop computes in FP32 where the reference does (operators, FastConvection, the products and the
vector updates; only the solves run in FP64 inside the library); the stepper in FP64.  The pressure
differs most because D u* cancels heavily and its FP32 sums leave rounding noise in the pressure
right-hand side.  Bounds: 10x the relative L2 differences measured on a GB300 (u 3.5e-6, p 4.6e-5).
"""

import os
import subprocess

import numpy as np
import pytest

from test_shims import build_loop

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _read(G, path):
    import ctypes as C
    info = (C.c_int * 2)()
    assert G.lib().nsf_io_vec_info(path.encode(), info) == 0
    v = np.zeros(info[0])
    assert G.lib().nsf_io_read_vec(path.encode(), v.ctypes.data_as(C.POINTER(C.c_double))) == 0
    return v


def test_shim_loop_matches_stepper(torch_cuda, channel_coarse, tmp_path):
    import nsfemoptim_gb300 as G
    prog = build_loop(str(tmp_path))
    up, pp = str(tmp_path / "u.vec"), str(tmp_path / "p.vec")
    r = subprocess.run([prog, channel_coarse, "1.2", "1e-3", "1e-3", "3", "pcg", "1e-8", "1e-8", up, pp],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    u, p = _read(G, up), _read(G, pp)
    ctx = G.build_chorin_context(G.load_gmsh(channel_coarse), 1.2)
    st = G.ChorinStepper(ctx, 1e-3, 1e-3, vel_method=1, vel_tol=1e-8, pres_tol=1e-8, vel_max_iters=1000,
                         pres_max_iters=20000, use_graph=False)
    st.step(3)
    us, ps = st.state()
    eu = np.linalg.norm(u - us) / np.linalg.norm(us)
    ep = np.linalg.norm(p - ps) / np.linalg.norm(ps)
    print(r.stdout)
    print(f"shim loop vs stepper: u {eu:.3e} p {ep:.3e}")
    assert eu <= 3.5e-5 and ep <= 4.6e-4, (eu, ep)

"""nsf_residual_noalloc (no device allocation during the call) against nsf_spmv, through the C ABI.

Two calls in a row on one stream: r must match nsf_spmv(a, x, y = b, -1, 1) within 1e-13 of
max |b| + max |A x| (the SpMV tolerance of the parity tests: the two kernels sum each row in a
different order) and the squared norms must match numpy on that r (relative 1e-12).  The second
call checks that the first left the static scratch ready for the next one.  nrhs outside
1..NSF_NOALLOC_MAX_RHS is rejected before anything runs on the device.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_RHS = 4  # NSF_NOALLOC_MAX_RHS in include/nsfem_gb300.h


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def system(torch_cuda, channel_coarse):
    import nsfemoptim_gb300 as G
    mesh = G.load_gmsh(channel_coarse)
    ctx = G.build_chorin_context(mesh, 1.2)
    m = ctx.matrix("M")  # P2 mass matrix: square, FP64
    return G, G.CsrF.from_host(m, dtype=G.NSF_F64), m


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_residual_noalloc_matches_spmv(system, torch_cuda):
    torch = torch_cuda
    G, a, m = system
    from nsfemoptim_gb300 import _lib
    L = _lib.lib()
    n = m.rows
    rng = np.random.default_rng(3)
    stream = torch.cuda.Stream()
    for nrhs in (1, 2, MAX_RHS):
        for call in range(2):  # two calls in a row
            x = torch.tensor(rng.standard_normal(nrhs * n), device="cuda")
            b = torch.tensor(rng.standard_normal(nrhs * n), device="cuda")
            r = torch.full((nrhs * n,), float("nan"), dtype=torch.float64, device="cuda")
            norms = torch.full((2 * nrhs,), float("nan"), dtype=torch.float64, device="cuda")
            with torch.cuda.stream(stream):
                st = L.nsf_residual_noalloc(a._h, nrhs, _ptr(x), _ptr(b), _ptr(r), _ptr(norms),
                                            C.c_void_p(stream.cuda_stream))
                assert st == 0, _lib.lib().nsf_last_error()
                # the existing entry point, channel by channel: y = -A x + y with y = b
                ref = b.clone()
                for c in range(nrhs):
                    yc = ref[c * n:(c + 1) * n]
                    xc = x[c * n:(c + 1) * n]
                    st = L.nsf_spmv(a._h, _ptr(xc), _ptr(yc), -1.0, 1.0, C.c_void_p(stream.cuda_stream))
                    assert st == 0
            stream.synchronize()
            scale = float(b.abs().max() + (ref - b).abs().max())
            assert float((r - ref).abs().max()) <= 1e-13 * scale, (nrhs, call)
            rh, bh = r.cpu().numpy(), b.cpu().numpy()
            want = [float(rh[c * n:(c + 1) * n] @ rh[c * n:(c + 1) * n]) for c in range(nrhs)] + \
                   [float(bh[c * n:(c + 1) * n] @ bh[c * n:(c + 1) * n]) for c in range(nrhs)]
            np.testing.assert_allclose(norms.cpu().numpy(), want, rtol=1e-12, atol=0)


def test_residual_noalloc_rejects_sizes(system, torch_cuda):
    torch = torch_cuda
    G, a, m = system
    from nsfemoptim_gb300 import _lib
    L = _lib.lib()
    n = m.rows
    big = MAX_RHS + 1
    x = torch.zeros(big * n, dtype=torch.float64, device="cuda")
    r = torch.zeros_like(x)
    norms = torch.zeros(2 * big, dtype=torch.float64, device="cuda")
    for bad in (0, big):
        st = L.nsf_residual_noalloc(a._h, bad, _ptr(x), _ptr(x), _ptr(r), _ptr(norms), None)
        assert st == _lib.NSF_ERR_INVALID_ARG
        assert b"outside" in L.nsf_last_error()
    # an FP32 matrix is refused too
    a32 = G.CsrF.from_host(m, dtype=G.NSF_F32)
    st = L.nsf_residual_noalloc(a32._h, 1, _ptr(x), _ptr(x), _ptr(r), _ptr(norms), None)
    assert st == _lib.NSF_ERR_INVALID_ARG

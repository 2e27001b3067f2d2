"""The SolverTest-compatible command-line tool and the headless frame dump on a GPU, through the C
ABI.

* nsf_solver_test solves systems written in the reference's binary format: the internal pressure
  stiffness of the committed channel mesh (float file, one channel, "cgCuda": CG with the multicolor
  SGS preconditioner to 1e-10 relative) and its velocity mass matrix with a two-channel interleaved
  right-hand side ("gaussSeidelCuda2": multicolor Gauss-Seidel, RMS target 1e-12).  Its iteration
  counts equal those of the same solves through the library, and its reported RMS residuals ("Final
  MSE", CsrMatrix::mse of the reference) meet the targets.
* nsf_chorin_dump writes the state as vector files that read back to nsf_chorin_get_state's values
  (FP64 exactly, FP32 as their rounding).
"""

import ctypes as C
import re
import subprocess

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
def ctx(torch_cuda, channel_coarse):
    import nsfemoptim_gb300 as G
    return G, G.build_chorin_context(G.load_gmsh(channel_coarse), 1.2)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _write(G, tmp_path, name, m, dtype, b):
    L = G.lib()
    mp, bp = str(tmp_path / f"{name}.csr"), str(tmp_path / f"{name}.vec")
    rs, ci = np.ascontiguousarray(m.rowStart, np.int32), np.ascontiguousarray(m.column, np.int32)
    v = np.ascontiguousarray(m.values, np.float64)
    assert L.nsf_io_write_csr(mp.encode(), m.rows, m.cols, m.nnz, _p(rs, C.c_int), _p(ci, C.c_int), _p(v, C.c_double),
                              dtype) == 0
    assert L.nsf_io_write_vec(bp.encode(), len(b), _p(np.ascontiguousarray(b), C.c_double), dtype) == 0
    return mp, bp


def _run(args):
    from nsfemoptim_gb300 import _build
    r = subprocess.run([_build.CLI] + args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_cli_cg_pressure(ctx, tmp_path, torch_cuda):
    G, c = ctx
    from nsfemoptim_gb300.api import HostCsr
    kpi = c.matrix("Kpi")
    b = np.random.default_rng(6).standard_normal(kpi.rows)
    mp, bp = _write(G, tmp_path, "kpi", kpi, 0, b)
    out = _run(["cgCuda", mp, bp, "2000", "1e-10"])
    assert "Single channel solve" in out
    it = int(re.search(r"Iterations = (\d+)", out).group(1))
    mse = float(re.search(r"Final MSE = (\S+)", out).group(1))
    # the same solve through the library, on the float-rounded system the file holds
    k32 = HostCsr(kpi.rows, kpi.cols, kpi.rowStart, kpi.column, kpi.values.astype(np.float32).astype(np.float64))
    b32 = b.astype(np.float32).astype(np.float64)
    s = G.create_solver("pcg", 1, k32, 2000, 1e-10, 1)
    s.getRhs().copy_(torch_cuda.tensor(b32))
    s.getSol().zero_()
    assert s.solve() == 0
    assert it == s.getLastIterations()
    assert mse <= 1.01e-10 * np.linalg.norm(b32) / np.sqrt(kpi.rows)
    assert re.search(r"Status = (\S+)", out).group(1) == G.lib().nsf_status_string(0).decode()


def test_cli_gs_two_channels(ctx, tmp_path):
    G, c = ctx
    m = c.matrix("M")
    n = m.rows
    rng = np.random.default_rng(7)
    planar = rng.standard_normal(2 * n)
    inter = np.empty(2 * n)
    inter[0::2], inter[1::2] = planar[:n], planar[n:]
    mp, bp = _write(G, tmp_path, "m", m, 1, inter)
    out = _run(["gaussSeidelCuda2", mp, bp, "200", "1e-12"])
    assert "Two channel solve" in out and "Number of channels = 2" in out
    a, bb = (float(v) for v in re.search(r"Final MSE = (\S+) / (\S+)", out).groups())
    assert a <= 1e-12 and bb <= 1e-12


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_chorin_dump_reads_back(ctx, tmp_path, dtype):
    G, c = ctx
    st = G.ChorinStepper(c, 1e-3, 1e-3, use_graph=False)
    st.step(3)
    u, p = st.state()
    up, pp = str(tmp_path / "u.vec"), str(tmp_path / "p.vec")
    code = G.NSF_F64 if dtype == "f64" else G.NSF_F32
    st.dump(up, pp, code)
    for path, ref in ((up, u), (pp, p)):
        info = (C.c_int * 2)()
        assert G.lib().nsf_io_vec_info(path.encode(), info) == 0
        assert list(info) == [len(ref), code]
        y = np.zeros(len(ref))
        assert G.lib().nsf_io_read_vec(path.encode(), _p(y, C.c_double)) == 0
        want = ref if dtype == "f64" else ref.astype(np.float32).astype(np.float64)
        assert np.array_equal(y, want)

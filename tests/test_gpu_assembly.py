"""On-device assembly (nsf_context_build_device) against the host assembly, through the C ABI.

The device kernels gather each output row over its incident elements in ascending order with the
host's operation order and explicitly rounded operations, so every value of M, K, Kp, Kpi, D, G and
the FastConvection matrix I equals the host's bit for bit, on the committed h = 0.025 mesh and the
reference's shipped h_0.01 mesh (where present); the boundary lists and patterns are the host's.
"""

import numpy as np
import pytest

from conftest import shipped_mesh_path

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("which", ["committed", "shipped_h0.01"])
def test_device_assembly_equals_host(torch_cuda, channel_coarse, which):
    import nsfemoptim_gb300 as G
    path = channel_coarse if which == "committed" else shipped_mesh_path("h_0.01.msh")
    if path is None:
        pytest.skip("shipped mesh not present")
    mesh = G.load_gmsh(path)
    host = G.build_chorin_context(mesh, 1.2)
    dev = G.build_chorin_context(mesh, 1.2, device=True)
    assert dev.assembly_ms is not None and dev.assembly_ms > 0
    assert np.array_equal(host.dir_ids, dev.dir_ids) and np.array_equal(host.dir_vx, dev.dir_vx)
    assert np.array_equal(host.int_p, dev.int_p)
    for name in G.ChorinContext.MATRICES:
        a, b = host.matrix(name), dev.matrix(name)
        assert np.array_equal(a.rowStart, b.rowStart) and np.array_equal(a.column, b.column), name
        assert np.array_equal(a.values, b.values), (name, np.abs(a.values - b.values).max())
    print(f"{which}: device assembly {dev.assembly_ms:.3f} ms")

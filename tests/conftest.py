import gzip
import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")

def _reference_assets():
    """The reference's shipped meshes (``cpp/assets``), where its tree is present."""
    import oracle
    root = oracle.reference_root()
    return os.path.join(root, "assets") if root else ""


REFERENCE_ASSETS = _reference_assets()
# copies of the shipped meshes made by the reference harness build (oracle/Makefile.ref)
HARNESS_ASSETS = os.path.join(ROOT, "oracle", "_ref", "assets")


def shipped_mesh_path(name):
    """Path of the reference's shipped mesh `name` (e.g. "h_0.01.msh"), from its tree or from the
    harness build's copy, or None."""
    for d in (REFERENCE_ASSETS, HARNESS_ASSETS):
        if d:
            p = os.path.join(d, name)
            if os.path.exists(p):
                return p
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


@pytest.fixture(scope="session")
def mesh_dir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("meshes"))


def _golden_mesh(name, mesh_dir):
    src = os.path.join(GOLDEN, name + ".msh.gz")
    dst = os.path.join(mesh_dir, name + ".msh")
    if not os.path.exists(dst):
        with gzip.open(src, "rb") as f, open(dst, "wb") as g:
            shutil.copyfileobj(f, g)
    return dst


@pytest.fixture(scope="session")
def channel_coarse(mesh_dir):
    """Committed synthetic DFG channel mesh, h = 0.025 (seed 0)."""
    return _golden_mesh("channel_h0.025_s0", mesh_dir)


@pytest.fixture(scope="session")
def square_small(mesh_dir):
    """Committed jittered unit square, 33 x 33 nodes (seed 0)."""
    return _golden_mesh("square_n33_s0", mesh_dir)


@pytest.fixture(scope="session")
def channel_h01(mesh_dir):
    """Synthetic DFG channel mesh at h = 0.01 generated from seed 0."""
    from nsfemoptim_gb300 import meshgen
    p = os.path.join(mesh_dir, "channel_h0.01_s0.msh")
    if not os.path.exists(p):
        meshgen.write_gmsh41(p, meshgen.dfg_channel(0.01, seed=0))
    return p


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

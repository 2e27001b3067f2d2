"""GB300-native (sm_103a) Chorin-projection path of a P2/P1 finite-element Navier-Stokes solver.

Host setup (gmsh input, numbering, FP64 assembly, coloring) is C++; the time step (FastConvection
SpMV, SpMM, multicolor Gauss-Seidel / SGS-preconditioned CG, projection) is hand-written CUDA in
``libnsfem_gb300.so`` behind the C ABI of ``include/nsfem_gb300.h``.  This package is the Python
mirror of that ABI; ``meshgen`` writes seeded synthetic meshes.
"""

from ._lib import NsfError, lib, LIB_PATH  # noqa: F401
from .api import *  # noqa: F401,F403
from . import meshgen  # noqa: F401

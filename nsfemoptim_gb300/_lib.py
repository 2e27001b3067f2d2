"""ctypes loader and signatures of libnsfem_gb300.so (the C ABI declared in include/nsfem_gb300.h).

The library is the only compute path: there is no CPU or vendor-library fallback.  Importing
this module never requires a GPU; calls that touch the device fail with NsfError(NSF_ERR_CUDA)
when none is present.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnsfem_gb300.so")

NSF_OK, NSF_ERR_INVALID_ARG, NSF_ERR_NONFINITE, NSF_ERR_MAXITER = 0, 1, 2, 3
NSF_ERR_BREAKDOWN, NSF_ERR_CUDA, NSF_ERR_IO, NSF_ERR_NOT_SUPPORTED = 4, 5, 6, 7
NSF_F32, NSF_F64 = 0, 1
NSF_PREC_F64, NSF_PREC_MIXED, NSF_PREC_F64_MIXEDSOLVE, NSF_PREC_MIXED_F32 = 0, 1, 2, 3
NSF_STATE_KEEP_HISTORY, NSF_STATE_ASYNC = 1, 2

i32p = C.POINTER(C.c_int)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
vp = C.c_void_p


class NsfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class ChorinConfig(C.Structure):
    _fields_ = [("nu", C.c_double), ("tau", C.c_double), ("precision", C.c_int), ("velMethod", C.c_int),
                ("velMaxIters", C.c_int), ("velTol", C.c_double), ("presMaxIters", C.c_int),
                ("presTol", C.c_double), ("checkInterval", C.c_int), ("useGraph", C.c_int),
                ("maxOuter", C.c_int), ("innerTol", C.c_double), ("pressureGuess", C.c_int),
                ("pressureBasis", C.c_int)]


class AdjointConfig(C.Structure):
    """nsf_adjoint_config"""
    _fields_ = [("checkpointInterval", C.c_int), ("maxIters", C.c_int), ("tol", C.c_double),
                ("snapshots", C.c_int)]


_SIGS = {
    "nsf_last_error": (C.c_char_p, []),
    "nsf_status_string": (C.c_char_p, [C.c_int]),
    "nsf_version": (C.c_int, []),
    "nsf_mesh_load_gmsh": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "nsf_mesh_counts": (C.c_int, [vp, i32p]),
    "nsf_mesh_arrays": (C.c_int, [vp, i32p, i32p, f32p, i32p]),
    "nsf_mesh_group": (C.c_char_p, [vp, C.c_int]),
    "nsf_mesh_destroy": (None, [vp]),
    "nsf_context_build": (C.c_int, [vp, C.c_float, C.c_int, C.POINTER(vp)]),
    "nsf_context_build_device": (C.c_int, [vp, C.c_float, C.c_int, C.POINTER(vp), f64p]),
    "nsf_context_sizes": (C.c_int, [vp, i32p]),
    "nsf_context_matrix": (C.c_int, [vp, C.c_int, i32p, i32p, f64p]),
    "nsf_context_lists": (C.c_int, [vp, i32p, f64p, i32p, i32p, i32p]),
    "nsf_context_destroy": (None, [vp]),
    "nsf_coloring": (C.c_int, [C.c_int, i32p, i32p, i32p, i32p, i32p]),
    "nsf_csr_create": (C.c_int, [C.c_int, C.c_int, C.c_int, i32p, i32p, vp, C.c_int, C.POINTER(vp)]),
    "nsf_csr_update_values": (C.c_int, [vp, vp, C.c_int, vp]),
    "nsf_csr_device": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "nsf_csr_destroy": (None, [vp]),
    "nsf_spmv": (C.c_int, [vp, vp, vp, C.c_double, C.c_double, vp]),
    "nsf_spmm": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, C.c_int, vp]),
    "nsf_fastconv_apply": (C.c_int, [vp, vp, C.c_double, vp, vp, vp]),
    "nsf_fastconv_apply_df": (C.c_int, [vp, vp, C.c_double, vp, vp, vp]),
    "nsf_residual_noalloc": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp]),
    "nsf_solver_create": (C.c_int, [C.c_char_p, C.c_int, C.c_int, i32p, i32p, f64p, C.c_int, C.c_int, C.c_double,
                                    C.c_int, C.POINTER(vp)]),
    "nsf_solver_solve": (C.c_int, [vp, vp, vp, vp]),
    "nsf_solver_solve_host": (C.c_int, [vp, f64p, f64p]),
    "nsf_solver_set_coarse": (C.c_int, [vp, C.POINTER(C.c_float), C.c_int]),
    "nsf_chorin_mass_solve": (C.c_int, [vp, C.c_void_p, C.c_void_p, C.c_double, C.POINTER(C.c_int), vp]),
    "nsf_solver_solve_f32": (C.c_int, [vp, vp, vp, vp]),
    "nsf_axpy": (C.c_int, [C.c_longlong, C.c_double, vp, vp, C.c_int, vp]),
    "nsf_scale": (C.c_int, [C.c_longlong, C.c_double, vp, C.c_int, vp]),
    "nsf_gather": (C.c_int, [C.c_int, vp, vp, vp, C.c_int, vp]),
    "nsf_scatter": (C.c_int, [C.c_int, vp, vp, vp, C.c_int, vp]),
    "nsf_solver_stats": (C.c_int, [vp, i32p, f64p, f64p]),
    "nsf_solver_set": (C.c_int, [vp, C.c_int, C.c_double, C.c_int]),
    "nsf_solver_destroy": (None, [vp]),
    "nsf_io_csr_info": (C.c_int, [C.c_char_p, i32p]),
    "nsf_io_read_csr": (C.c_int, [C.c_char_p, i32p, i32p, f64p]),
    "nsf_io_write_csr": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, i32p, i32p, f64p, C.c_int]),
    "nsf_io_vec_info": (C.c_int, [C.c_char_p, i32p]),
    "nsf_io_read_vec": (C.c_int, [C.c_char_p, f64p]),
    "nsf_io_write_vec": (C.c_int, [C.c_char_p, C.c_int, f64p, C.c_int]),
    "nsf_chorin_dump": (C.c_int, [vp, C.c_char_p, C.c_char_p, C.c_int, vp]),
    "nsf_batch_create": (C.c_int, [vp, C.POINTER(ChorinConfig), C.c_int, f64p, f64p, C.POINTER(vp)]),
    "nsf_batch_step": (C.c_int, [vp, C.c_int, vp]),
    "nsf_batch_launch": (C.c_int, [vp, C.c_int, vp]),
    "nsf_batch_get_state": (C.c_int, [vp, C.c_int, f64p, f64p, vp]),
    "nsf_batch_set_state": (C.c_int, [vp, C.c_int, f64p, f64p, vp]),
    "nsf_batch_stats": (C.c_int, [vp, C.c_int, f64p]),
    "nsf_batch_kernels_per_step": (C.c_longlong, [vp]),
    "nsf_batch_destroy": (None, [vp]),
    "nsf_neumann_create": (C.c_int, [C.c_int, i32p, i32p, f64p, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.POINTER(vp)]),
    "nsf_neumann_solve": (C.c_int, [vp, vp, vp, vp]),
    "nsf_neumann_stats": (C.c_int, [vp, i32p, f64p]),
    "nsf_neumann_destroy": (None, [vp]),
    "nsf_chorin_create": (C.c_int, [vp, C.POINTER(ChorinConfig), C.POINTER(vp)]),
    "nsf_chorin_step": (C.c_int, [vp, C.c_int, vp]),
    "nsf_chorin_launch": (C.c_int, [vp, C.c_int, vp]),
    "nsf_chorin_get_state": (C.c_int, [vp, f64p, f64p, vp]),
    "nsf_chorin_set_state": (C.c_int, [vp, f64p, f64p, vp]),
    "nsf_chorin_set_state_ex": (C.c_int, [vp, f64p, f64p, C.c_int, vp]),
    "nsf_chorin_stats": (C.c_int, [vp, f64p]),
    "nsf_kernel_launches": (C.c_longlong, []),
    "nsf_chorin_destroy": (None, [vp]),
    "nsf_forces_create": (C.c_int, [vp, vp, C.c_char_p, C.POINTER(vp)]),
    "nsf_forces_eval": (C.c_int, [vp, vp, C.c_int, vp]),
    "nsf_forces_destroy": (None, [vp]),
    "nsf_chorin_set_dirichlet": (C.c_int, [vp, f64p, vp]),
    "nsf_chorin_set_nu": (C.c_int, [vp, C.c_double]),
    "nsf_adjoint_create": (C.c_int, [vp, vp, C.POINTER(AdjointConfig), C.POINTER(vp)]),
    "nsf_adjoint_run": (C.c_int, [vp, C.c_int, f64p, f64p, f64p, f64p, f64p, vp]),
    "nsf_adjoint_stats": (C.c_int, [vp, f64p]),
    "nsf_adjoint_destroy": (None, [vp]),
    "nsf_pack_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(vp)]),
    "nsf_pack_create_batches": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(vp)]),
    "nsf_pack_kernels_per_step": (C.c_longlong, [vp]),
    "nsf_pack_step": (C.c_int, [vp, C.c_int, vp]),
    "nsf_pack_destroy": (None, [vp]),
}

_LIB = None


def lib():
    """Load libnsfem_gb300.so, building it in-tree on first use if it is missing."""
    global _LIB
    if _LIB is None:
        path = os.environ.get("NSF_LIBRARY") or LIB_PATH  # an alternative build of the same ABI
        if path == LIB_PATH and not os.path.exists(LIB_PATH):
            from . import _build
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(status: int) -> None:
    if status != NSF_OK:
        msg = lib().nsf_last_error()
        raise NsfError(status, msg.decode() if msg else lib().nsf_status_string(status).decode())


def declared_symbols() -> list:
    return list(_SIGS.keys())

"""Python mirror of the reference's matrix/solver interface over the C ABI.

Names, argument meaning and error behaviour follow the reference's ``cu::`` classes
(``cpp/libs/CudaUtils/include/cu/``) and setup functions:

* ``load_gmsh``                  mesh::parseTriangleGmsh + mesh::createMesh (P2 and P1)
* ``build_chorin_context``       buildChorinContext (cpp/execs/NavierStokes/src/buildContext.cpp:17)
* ``CsrF``                       cu::csrF (device CSR; FP64 or FP32 values)
* ``Spmv`` / ``Spmm``            cu::spmv / cu::spmm (default x/b members, ``compute()``)
* ``create_solver``              cu::createSolver returning an ``AbstractSolver`` with
                                 getNumCh / getLastMse / getLastIterations / getRhs / getSol /
                                 solve / setMaxIters / setTargetMse / setMseCheckInterval
* ``ChorinStepper``              the device time loop of solveNsChorinCuda

Device vectors are torch CUDA tensors (used only as device memory); failures raise NsfError
with the library's status code, as the reference throws std::runtime_error.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (NSF_F32, NSF_F64, NSF_PREC_F64, NSF_PREC_F64_MIXEDSOLVE, NSF_PREC_MIXED, NSF_PREC_MIXED_F32,
                   NSF_STATE_ASYNC, NSF_STATE_KEEP_HISTORY, ChorinConfig, NsfError, check, lib, vp)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _dptr(t):
    return C.c_void_p(int(t.data_ptr()))


def _torch():
    import torch
    return torch


# ------------------------------------------------------------------------------------ host setup

class Mesh:
    """P2 velocity / P1 pressure mesh read from a gmsh MSH 4.1 file."""

    def __init__(self, path: str):
        h = vp()
        check(lib().nsf_mesh_load_gmsh(path.encode(), C.byref(h)))
        self._h = h
        c = (C.c_int * 6)()
        check(lib().nsf_mesh_counts(h, c))
        self.num_corner, self.num_tri, self.num_border, self.N, self.P, n_groups = list(c)
        self.groups = [lib().nsf_mesh_group(h, i).decode() for i in range(n_groups)]

    def pressure_xy(self):
        """(P, 2) coordinates of the P1 (pressure) nodes: the element corners, P2 nodes 0, 2, 4."""
        v_elem, p_elem, v_xy, _ = self.arrays()
        xy = np.zeros((self.P, 2), np.float32)
        xy[p_elem.ravel()] = v_xy[v_elem[:, 0::2].ravel()]
        return xy

    def arrays(self):
        T, B = self.num_tri, self.num_border
        v_elem = np.zeros(6 * T, np.int32)
        p_elem = np.zeros(3 * T, np.int32)
        v_xy = np.zeros(2 * self.N, np.float32)
        v_border = np.zeros(6 * B, np.int32)
        check(lib().nsf_mesh_arrays(self._h, _p(v_elem, C.c_int), _p(p_elem, C.c_int), _p(v_xy, C.c_float),
                                    _p(v_border, C.c_int)))
        return v_elem.reshape(T, 6), p_elem.reshape(T, 3), v_xy.reshape(-1, 2), v_border.reshape(B, 6)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_mesh_destroy(self._h)
            self._h = None


def load_gmsh(path: str) -> Mesh:
    return Mesh(path)


class HostCsr:
    def __init__(self, rows, cols, rowStart, column, values):
        self.rows, self.cols = rows, cols
        self.rowStart, self.column, self.values = rowStart, column, values

    @property
    def nnz(self):
        return int(self.column.shape[0])


class ChorinContext:
    """Boundary lists and FP64 operators of the channel problem (fem::ChorinContextF)."""

    MATRICES = ("M", "K", "Kp", "Kpi", "D", "G", "I")

    def __init__(self, mesh: Mesh, peak_velocity: float, n_threads: int = 0, device: bool = False):
        """device: assemble the operator values on the GPU (nsf_context_build_device; the same bits)."""
        h = vp()
        self.assembly_ms = None
        if device:
            ms = C.c_double(0.0)
            check(lib().nsf_context_build_device(mesh._h, C.c_float(peak_velocity), n_threads, C.byref(h),
                                                 C.byref(ms)))
            self.assembly_ms = ms.value
        else:
            check(lib().nsf_context_build(mesh._h, C.c_float(peak_velocity), n_threads, C.byref(h)))
        self._h = h
        s = (C.c_int * 13)()
        check(lib().nsf_context_sizes(h, s))
        s = list(s)
        self.N, self.P, n_dir, n_dir_p, n_int_v, n_int_p = s[:6]
        self._nnz = dict(zip(self.MATRICES, s[6:]))
        self.dir_ids = np.zeros(n_dir, np.int32)
        self.dir_vx = np.zeros(n_dir, np.float64)
        self.dir_p_ids = np.zeros(n_dir_p, np.int32)
        self.int_v = np.zeros(n_int_v, np.int32)
        self.int_p = np.zeros(n_int_p, np.int32)
        check(lib().nsf_context_lists(h, _p(self.dir_ids, C.c_int), _p(self.dir_vx, C.c_double),
                                      _p(self.dir_p_ids, C.c_int), _p(self.int_v, C.c_int),
                                      _p(self.int_p, C.c_int)))
        self._cache = {}

    def _shape(self, name):
        N, P, nip = self.N, self.P, len(self.int_p)
        return {"M": (N, N), "K": (N, N), "Kp": (P, P), "Kpi": (nip, nip), "D": (P, 2 * N), "G": (2 * N, P),
                "I": (self._nnz["K"], 2 * N)}[name]

    def matrix(self, name: str) -> HostCsr:
        if name not in self._cache:
            rows, cols = self._shape(name)
            nnz = self._nnz[name]
            rs = np.zeros(rows + 1, np.int32)
            ci = np.zeros(nnz, np.int32)
            va = np.zeros(nnz, np.float64)
            check(lib().nsf_context_matrix(self._h, self.MATRICES.index(name), _p(rs, C.c_int), _p(ci, C.c_int),
                                           _p(va, C.c_double)))
            self._cache[name] = HostCsr(rows, cols, rs, ci, va)
        return self._cache[name]

    def __getattr__(self, name):
        if name in ChorinContext.MATRICES:
            return self.matrix(name)
        raise AttributeError(name)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_context_destroy(self._h)
            self._h = None


def build_chorin_context(mesh: Mesh, peak_velocity: float, n_threads: int = 0, device: bool = False) -> ChorinContext:
    return ChorinContext(mesh, peak_velocity, n_threads, device)


def coloring(rowStart, column):
    """(perm, partStart) of the smallest-last + greedy coloring (cu::GaussSeidel's ordering)."""
    rs, ci = _i32(rowStart), _i32(column)
    n = len(rs) - 1
    perm = np.zeros(n, np.int32)
    part = np.zeros(n + 1, np.int32)
    nc = C.c_int(0)
    check(lib().nsf_coloring(n, _p(rs, C.c_int), _p(ci, C.c_int), _p(perm, C.c_int), _p(part, C.c_int),
                             C.byref(nc)))
    return perm, part[: nc.value + 1].copy()


# ------------------------------------------------------------------------------------ device CSR

class CsrF:
    """Device CSR (cu::csrF).  ``values`` are FP64 or FP32 (``dtype``)."""

    def __init__(self, rows, cols, rowStart, column, values, dtype=NSF_F64):
        self.rows, self.cols = int(rows), int(cols)
        rs, ci = _i32(rowStart), _i32(column)
        self.nnz = int(ci.shape[0])
        self.dtype = dtype
        va = np.ascontiguousarray(values, dtype=np.float64 if dtype == NSF_F64 else np.float32)
        h = vp()
        check(lib().nsf_csr_create(self.rows, self.cols, self.nnz, _p(rs, C.c_int), _p(ci, C.c_int),
                                   va.ctypes.data_as(vp), dtype, C.byref(h)))
        self._h = h

    @staticmethod
    def from_host(a: HostCsr, dtype=NSF_F64) -> "CsrF":
        return CsrF(a.rows, a.cols, a.rowStart, a.column, a.values, dtype)

    @property
    def torch_dtype(self):
        t = _torch()
        return t.float64 if self.dtype == NSF_F64 else t.float32

    def update_values(self, values, stream=None):
        t = _torch()
        if isinstance(values, t.Tensor) and values.is_cuda:
            check(lib().nsf_csr_update_values(self._h, _dptr(values), 1, vp(stream)))
        else:
            va = np.ascontiguousarray(values, dtype=np.float64 if self.dtype == NSF_F64 else np.float32)
            check(lib().nsf_csr_update_values(self._h, va.ctypes.data_as(vp), 0, vp(stream)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_csr_destroy(self._h)
            self._h = None


def spmv(a: CsrF, x, y, alpha=1.0, beta=0.0, stream=None):
    check(lib().nsf_spmv(a._h, _dptr(x), _dptr(y), alpha, beta, vp(stream)))
    return y


def spmm(a: CsrF, X, Y, nrhs: int, stream=None):
    check(lib().nsf_spmm(a._h, nrhs, _dptr(X), a.cols, _dptr(Y), a.rows, vp(stream)))
    return Y


def fastconv_apply(I: CsrF, K_values, nu: float, u, A_values, stream=None):
    """A = nu * K + I u (the reference's FastConvection SpMV followed by the Sgeam add)."""
    check(lib().nsf_fastconv_apply(I._h, _dptr(K_values), nu, _dptr(u), _dptr(A_values), vp(stream)))
    return A_values


def fastconv_apply_df(I: CsrF, K_values, nu: float, u, A_values, stream=None):
    """A = nu * K + I u with I in FP32 and K, u, A (and the sums) as double-floats: float32 device
    tensors of shape (n, 2) holding (hi, lo), value = hi + lo.  The mixed stepper's FastConvection
    product."""
    check(lib().nsf_fastconv_apply_df(I._h, _dptr(K_values), nu, _dptr(u), _dptr(A_values), vp(stream)))
    return A_values


def split_df(x):
    """(n, 2) float32 (hi, lo) pairs of an FP64 array (numpy or torch), value = hi + lo."""
    if isinstance(x, np.ndarray):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
        return np.stack([hi, lo], axis=1)
    import torch
    hi = x.float()
    lo = (x - hi.double()).float()
    return torch.stack([hi, lo], dim=1).contiguous()


class Spmv:
    """cu::spmv: b = M x with default operand vectors."""

    def __init__(self, mat: CsrF):
        t = _torch()
        self.mat = mat
        self.x = t.zeros(mat.cols, dtype=mat.torch_dtype, device="cuda")
        self.b = t.zeros(mat.rows, dtype=mat.torch_dtype, device="cuda")

    def compute(self, x=None, b=None):
        return spmv(self.mat, self.x if x is None else x, self.b if b is None else b)


class Spmm:
    """cu::spmm: planar multi-channel b = M x."""

    def __init__(self, mat: CsrF, numCh: int):
        t = _torch()
        self.mat, self.numCh = mat, numCh
        self.x = t.zeros(mat.cols * numCh, dtype=mat.torch_dtype, device="cuda")
        self.b = t.zeros(mat.rows * numCh, dtype=mat.torch_dtype, device="cuda")

    def compute(self, x=None, b=None):
        return spmm(self.mat, self.x if x is None else x, self.b if b is None else b, self.numCh)


# ------------------------------------------------------------------------------------ solvers

class AbstractSolver:
    """cu::AbstractSolver over nsf_solver.  getRhs()/getSol() are the device IO vectors; getSol()
    is also the initial guess (zero it before solve() for a cold start, as the reference's callers
    do)."""

    def __init__(self, name, numCh, m: HostCsr, maxIters, targetMse, mseCheckInterval, precision=NSF_PREC_F64):
        t = _torch()
        if m.rows != m.cols:
            raise NsfError(1, "matrix must be square")
        h = vp()
        rs, ci = _i32(m.rowStart), _i32(m.column)
        va = np.ascontiguousarray(m.values, dtype=np.float64)
        check(lib().nsf_solver_create(name.encode(), numCh, m.rows, _p(rs, C.c_int), _p(ci, C.c_int),
                                      _p(va, C.c_double), precision, maxIters, targetMse, mseCheckInterval,
                                      C.byref(h)))
        self._h = h
        self.name, self.numCh, self.n = name, numCh, m.rows
        self.maxIters, self.targetMse, self.mseCheckInterval = maxIters, targetMse, mseCheckInterval
        self._rhs = t.zeros(numCh * m.rows, dtype=t.float64, device="cuda")
        self._sol = t.zeros(numCh * m.rows, dtype=t.float64, device="cuda")
        self.last_status = 0

    def getNumCh(self):
        return self.numCh

    def setCoarse(self, xy, rows_per_aggregate: int = 240):
        """Two-level preconditioner (nsf_solver_set_coarse): xy are the coordinates of the rows
        ((rows, 2) array), the aggregates mesh cells of about rows_per_aggregate rows."""
        xy = np.ascontiguousarray(xy, dtype=np.float32).reshape(-1)
        check(lib().nsf_solver_set_coarse(self._h, _p(xy, C.c_float), int(rows_per_aggregate)))

    def getRhs(self):
        return self._rhs

    def getSol(self):
        return self._sol

    def solve(self, raise_on_status: bool = False):
        st = lib().nsf_solver_solve(self._h, _dptr(self._rhs), _dptr(self._sol), None)
        self.last_status = st
        if st != 0 and (raise_on_status or st not in (2, 3, 4)):
            check(st)
        return st

    def _stats(self):
        it = C.c_int(0)
        rms = (C.c_double * self.numCh)()
        rel = (C.c_double * self.numCh)()
        check(lib().nsf_solver_stats(self._h, C.byref(it), rms, rel))
        return it.value, list(rms), list(rel)

    def getLastMse(self, ch: int = -1):
        _, rms, _ = self._stats()
        if ch < 0:
            return float(np.sqrt(np.sum(np.square(rms))))
        return rms[ch] if ch < self.numCh else -1.0

    def getLastRelativeResidual(self, ch: int = 0):
        return self._stats()[2][ch]

    def getLastIterations(self):
        return self._stats()[0]

    def setMaxIters(self, n):
        self.maxIters = n
        check(lib().nsf_solver_set(self._h, self.maxIters, self.targetMse, self.mseCheckInterval))

    def setTargetMse(self, mse):
        self.targetMse = mse
        check(lib().nsf_solver_set(self._h, self.maxIters, self.targetMse, self.mseCheckInterval))

    def setMseCheckInterval(self, k):
        if k < 1:
            raise NsfError(1, "MSE check interval should be at least 1")
        self.mseCheckInterval = k
        check(lib().nsf_solver_set(self._h, self.maxIters, self.targetMse, self.mseCheckInterval))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_solver_destroy(self._h)
            self._h = None


class Batch:
    """Batched instances on one mesh (nsf_batch_*): instance q has viscosity nus[q] and Dirichlet x
    values dir_vx[q] (context dirIds order; None: the context's inflow for all), every operation of
    the time step one launch for all instances.  Mixed precision, Chebyshev mass solves, any pressure
    guess (2: one projection basis per instance); each instance computes what a ChorinStepper with
    the same options computes."""

    def __init__(self, ctx: ChorinContext, nus, tau: float, dir_vx=None, vel_max_iters: int = 500,
                 vel_tol: float = 1e-8, pres_max_iters: int = 5000, pres_tol: float = 1e-8, use_graph: bool = True,
                 max_outer: int = 4, inner_tol: float = 1e-5, pressure_guess: int = 2, pressure_basis: int = 0):
        self.ctx = ctx
        nus = np.ascontiguousarray(nus, dtype=np.float64)
        self.B = len(nus)
        self.cfg = ChorinConfig(float(nus[0]), tau, NSF_PREC_MIXED, 3, vel_max_iters, vel_tol, pres_max_iters,
                                pres_tol, 8, int(use_graph), max_outer, inner_tol, int(pressure_guess),
                                int(pressure_basis))
        dv = None
        if dir_vx is not None:
            dv = np.ascontiguousarray(dir_vx, dtype=np.float64).reshape(self.B, -1)
        h = vp()
        check(lib().nsf_batch_create(ctx._h, C.byref(self.cfg), self.B, _p(nus, C.c_double),
                                     _p(dv, C.c_double) if dv is not None else None, C.byref(h)))
        self._h = h
        self.N, self.P = ctx.N, ctx.P

    def step(self, n: int = 1, stream=None):
        check(lib().nsf_batch_step(self._h, n, vp(stream)))

    def launch(self, n: int = 1, stream=None):
        check(lib().nsf_batch_launch(self._h, n, vp(stream)))

    def state(self, q: int):
        u = np.zeros(2 * self.N, np.float64)
        p = np.zeros(self.P, np.float64)
        check(lib().nsf_batch_get_state(self._h, q, _p(u, C.c_double), _p(p, C.c_double), None))
        return u, p

    def set_state(self, q: int, u, p):
        u = np.ascontiguousarray(u, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        check(lib().nsf_batch_set_state(self._h, q, _p(u, C.c_double), _p(p, C.c_double), None))

    def stats(self, q: int):
        s = (C.c_double * 4)()
        check(lib().nsf_batch_stats(self._h, q, s))
        return {"pres_iters": s[0], "pres_rel": s[1], "replacements": s[2], "status": s[3]}

    def kernels_per_step(self) -> int:
        return int(lib().nsf_batch_kernels_per_step(self._h))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_batch_destroy(self._h)
            self._h = None


class NeumannSolver:
    """Pure-Neumann Poisson solve made regular by one Dirichlet pin (nsf_neumann_*): on the device, the
    right-hand side is projected to zero mean, the system without row/column `pin` is solved with
    the "pcg" solver, and the solution is expanded (x[pin] = 0) and shifted to zero mean, in FP64.
    solve(b, x): device FP64 tensors of n entries, x the initial guess."""

    def __init__(self, m: HostCsr, pin: int = 0, precision: int = NSF_PREC_F64, max_iters: int = 20000,
                 target: float = 1e-10):
        if m.rows != m.cols:
            raise NsfError(1, "matrix must be square")
        h = vp()
        rs, ci = _i32(m.rowStart), _i32(m.column)
        va = np.ascontiguousarray(m.values, dtype=np.float64)
        check(lib().nsf_neumann_create(m.rows, _p(rs, C.c_int), _p(ci, C.c_int), _p(va, C.c_double), int(pin),
                                       precision, max_iters, target, C.byref(h)))
        self._h, self.n, self.pin = h, m.rows, pin

    def solve(self, b, x, stream=None):
        return check(lib().nsf_neumann_solve(self._h, _dptr(b), _dptr(x), stream))

    def stats(self):
        it = C.c_int(0)
        rel = C.c_double(0.0)
        check(lib().nsf_neumann_stats(self._h, C.byref(it), C.byref(rel)))
        return {"iters": it.value, "rel": rel.value}

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_neumann_destroy(self._h)
            self._h = None


def create_solver(name: str, numCh: int, m: HostCsr, maxIters: int, targetMse: float, mseCheckInterval: int,
                  precision: int = NSF_PREC_F64) -> AbstractSolver:
    """cu::createSolver: "gs" (multicolor Gauss-Seidel, absolute RMS target) or "pcg" (CG with the
    multicolor symmetric Gauss-Seidel preconditioner, relative target)."""
    if numCh < 1:
        raise NsfError(1, f"Invalid number of channels for solver: {numCh}")
    if mseCheckInterval < 1:
        raise NsfError(1, f"Invalid MSE check interval for solver: {mseCheckInterval}")
    if name not in ("gs", "pcg"):
        raise NsfError(1, f"Invalid solver name: {name}")
    return AbstractSolver(name, numCh, m, maxIters, targetMse, mseCheckInterval, precision)


# ------------------------------------------------------------------------------------ stepper

class ChorinStepper:
    """Device-resident Chorin projection time stepper (the loop of solveNsChorinCuda)."""

    def __init__(self, ctx: ChorinContext, nu: float, tau: float, precision: int = NSF_PREC_F64,
                 vel_method: int = 1, vel_max_iters: int = 200, vel_tol: float = 1e-10,
                 pres_max_iters: int = 2000, pres_tol: float = 1e-10, check_interval: int = 8,
                 use_graph: bool = True, max_outer: int = 4, inner_tol: float = 1e-4, pressure_guess: int = 0,
                 pressure_basis: int = 0):
        """vel_method: mass solve, 0 multicolor GS, 1 PCG-SGS, 2 PCG-Jacobi, 3 Chebyshev-Jacobi,
        4 Chebyshev-Jacobi warm-started from the previous step's solution.
        pressure_guess: 0 the previous pressure (as the reference), 1 extrapolated from the last two,
        2 projected onto up to pressure_basis earlier solutions (0: 250)."""
        self.ctx = ctx
        self.cfg = ChorinConfig(nu, tau, precision, vel_method, vel_max_iters, vel_tol, pres_max_iters, pres_tol,
                                check_interval, int(use_graph), max_outer, inner_tol, int(pressure_guess),
                                int(pressure_basis))
        h = vp()
        check(lib().nsf_chorin_create(ctx._h, C.byref(self.cfg), C.byref(h)))
        self._h = h
        self.N, self.P = ctx.N, ctx.P

    def step(self, n: int = 1, stream=None):
        check(lib().nsf_chorin_step(self._h, n, vp(stream)))

    def launch(self, n: int = 1, stream=None):
        """Enqueue n steps (graph replays) without waiting: independent steppers on their own
        streams advance concurrently.  stats() keeps the last step() call's statistics."""
        check(lib().nsf_chorin_launch(self._h, n, vp(stream)))

    def state(self):
        u = np.zeros(2 * self.N, np.float64)
        p = np.zeros(self.P, np.float64)
        check(lib().nsf_chorin_get_state(self._h, _p(u, C.c_double), _p(p, C.c_double), None))
        return u, p

    def get_state_into(self, u: np.ndarray, p: np.ndarray, stream=None):
        """The state into u (2N) and p (P), float64 arrays; returns when they are written."""
        check(lib().nsf_chorin_get_state(self._h, _p(u, C.c_double), _p(p, C.c_double), vp(stream)))

    def set_state(self, u, p, keep_history: bool = False, asynchronous: bool = False, stream=None):
        """keep_history: the state continues this stepper's run, so the pressure-guess history is
        kept (otherwise a new one starts); only the initial guesses differ.  asynchronous
        (NSF_STATE_ASYNC): the copies are enqueued on the stream and the call returns at once; u and
        p must then be C-contiguous float64 arrays (no temporary copies), best in page-locked
        memory, left unchanged until the stream has passed them."""
        if asynchronous:
            for a in (u, p):
                if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]):
                    raise ValueError("asynchronous set_state needs C-contiguous float64 arrays")
        else:
            u = np.ascontiguousarray(u, np.float64)
            p = np.ascontiguousarray(p, np.float64)
        flags = (NSF_STATE_KEEP_HISTORY if keep_history else 0) | (NSF_STATE_ASYNC if asynchronous else 0)
        check(lib().nsf_chorin_set_state_ex(self._h, _p(u, C.c_double), _p(p, C.c_double), flags, vp(stream)))

    def dump(self, u_path=None, p_path=None, dtype=NSF_F64):
        """Headless frame output (nsf_chorin_dump): u (2N, planar) and p (P) in the original numbering
        to vector files of the reference's binary format, as float (NSF_F32) or double (NSF_F64)."""
        check(lib().nsf_chorin_dump(self._h, u_path.encode() if u_path else None,
                                    p_path.encode() if p_path else None, dtype, None))

    def set_dirichlet(self, dir_vx, stream=None):
        """Replace the x values of the Dirichlet velocity nodes (ctx.dir_ids order) and impose them
        on the current state.  New: the reference fixes the inflow for a run."""
        d = np.ascontiguousarray(dir_vx, np.float64)
        if d.shape != (len(self.ctx.dir_ids),):
            raise NsfError(1, "one Dirichlet value per Dirichlet node")
        check(lib().nsf_chorin_set_dirichlet(self._h, _p(d, C.c_double), vp(stream)))

    def set_nu(self, nu: float):
        """Viscosity of the following steps."""
        check(lib().nsf_chorin_set_nu(self._h, float(nu)))
        self.cfg.nu = float(nu)

    def mass_solve(self, b, x, tol: float = 1e-8, stream=None):
        """M x = b with the stepper's Chebyshev mass solve (velMethod 3); b, x: CUDA FP64 tensors of
        2 N entries in the stepper's numbering.  Returns the iterations run.  Shares the tentative
        mass solve's work buffers: not concurrently with this stepper's steps."""
        it = C.c_int(0)
        check(lib().nsf_chorin_mass_solve(self._h, _dptr(b), _dptr(x), float(tol), C.byref(it), vp(stream)))
        return it.value

    def stats(self):
        s = (C.c_double * 8)()
        check(lib().nsf_chorin_stats(self._h, s))
        keys = ("tent_iters", "pres_iters", "final_iters", "pres_rel", "tent_rel", "final_rel", "pres_passes",
                "status")
        return dict(zip(keys, list(s)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_chorin_destroy(self._h)
            self._h = None


def kernel_launches() -> int:
    return int(lib().nsf_kernel_launches())


class Forces:
    """Drag/lift functional on a border group ("Circle": the cylinder) of a stepper's state:
    F = integral (-p n + nu du/dn) ds, n into the fluid, FP64 on the device.  New: the reference
    has no force functional."""

    def __init__(self, mesh: Mesh, stepper: ChorinStepper, group: str = "Circle"):
        h = vp()
        check(lib().nsf_forces_create(mesh._h, stepper._h, group.encode(), C.byref(h)))
        self._h = h
        self._stepper = stepper  # the stepper must outlive the functional

    def __call__(self, stream=None) -> np.ndarray:
        """(F_x, F_y) of the current state (synchronous)."""
        out = np.zeros(2, np.float64)
        check(lib().nsf_forces_eval(self._h, _p(out, C.c_double), 0, vp(stream)))
        return out

    def into(self, out, stream=None):
        """Write (F_x, F_y) into a device tensor of 2 doubles, asynchronously on stream."""
        check(lib().nsf_forces_eval(self._h, _dptr(out), 1, vp(stream)))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_forces_destroy(self._h)
            self._h = None


class Pack:
    """Steppers advanced together by one CUDA graph launch per step (each stepper's time step is a
    branch of the graph).  New: the reference drives one flow.  With more than one stepper, create
    them with NSF_PCG_PATH=auto-cluster in the environment (solves inside thread-block clusters)."""

    def __init__(self, steppers):
        """steppers: ChorinStepper objects, or Batch objects (one graph branch per batch)."""
        self._steppers = list(steppers)  # they must outlive the pack
        arr = (vp * len(self._steppers))(*[s._h for s in self._steppers])
        h = vp()
        if all(isinstance(s, Batch) for s in self._steppers):
            check(lib().nsf_pack_create_batches(arr, len(self._steppers), C.byref(h)))
        else:
            check(lib().nsf_pack_create(arr, len(self._steppers), C.byref(h)))
        self._h = h

    def kernels_per_step(self) -> int:
        return int(lib().nsf_pack_kernels_per_step(self._h))

    def step(self, n: int = 1, stream=None):
        """Enqueue n graph launches (asynchronous)."""
        check(lib().nsf_pack_step(self._h, int(n), vp(stream)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_pack_destroy(self._h)
            self._h = None


class Adjoint:
    """Discrete adjoint of an FP64 stepper's time step for the force functional of `forces`:
    J = sum_n w_drag[n] F_x(u_n, p_n) + w_lift[n] F_y(u_n, p_n).  New: the reference has no adjoint.

    checkpoint_interval: steps between stored states (segments recomputed in the reverse sweep);
    0 keeps every state.  snapshots > 0: binomial checkpointing with at most that many stored
    states besides the initial one (checkpoint_interval ignored)."""

    STATS = ("forward_steps", "recomputed_steps", "reverse_steps", "mass_iters", "pres_iters",
             "forward_status", "adjoint_status", "state_bytes", "forward_ms", "reverse_ms")

    def __init__(self, stepper: ChorinStepper, forces: Forces, checkpoint_interval: int = 50,
                 max_iters: int = 20000, tol: float = 1e-13, snapshots: int = 0):
        from ._lib import AdjointConfig
        self.cfg = AdjointConfig(int(checkpoint_interval), int(max_iters), float(tol), int(snapshots))
        h = vp()
        check(lib().nsf_adjoint_create(stepper._h, forces._h, C.byref(self.cfg), C.byref(h)))
        self._h = h
        self._keep = (stepper, forces)
        self.N = stepper.N
        self.n_dir = len(stepper.ctx.dir_ids)

    def run(self, n_steps: int, w_drag=None, w_lift=None, stream=None):
        """Forward n_steps from the stepper's state, then the reverse sweep.
        Returns (J, dJ/dnu, dJ/d dirVx [nDir], dJ/du0 [2N])."""
        wd = np.ascontiguousarray(np.broadcast_to(np.asarray(0.0 if w_drag is None else w_drag, np.float64),
                                                  (n_steps,)))
        wl = np.ascontiguousarray(np.broadcast_to(np.asarray(0.0 if w_lift is None else w_lift, np.float64),
                                                  (n_steps,)))
        res = np.zeros(2, np.float64)
        gd = np.zeros(max(1, self.n_dir), np.float64)
        gu = np.zeros(2 * self.N, np.float64)
        check(lib().nsf_adjoint_run(self._h, int(n_steps), _p(wd, C.c_double), _p(wl, C.c_double),
                                    _p(res, C.c_double), _p(gd, C.c_double), _p(gu, C.c_double), vp(stream)))
        return float(res[0]), float(res[1]), gd[:self.n_dir].copy(), gu

    def stats(self):
        s = (C.c_double * 10)()
        check(lib().nsf_adjoint_stats(self._h, s))
        return dict(zip(self.STATS, list(s)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nsf_adjoint_destroy(self._h)
            self._h = None


__all__ = ["Mesh", "load_gmsh", "ChorinContext", "build_chorin_context", "coloring", "CsrF", "Spmv", "Spmm",
           "NeumannSolver", "Batch",
           "spmv", "spmm", "fastconv_apply", "fastconv_apply_df", "split_df", "AbstractSolver", "create_solver", "ChorinStepper", "kernel_launches",
           "Forces", "Adjoint", "Pack", "NSF_F32", "NSF_F64", "NSF_PREC_F64", "NSF_PREC_MIXED", "NSF_PREC_F64_MIXEDSOLVE", "NSF_PREC_MIXED_F32",
           "NSF_STATE_KEEP_HISTORY", "NSF_STATE_ASYNC", "NsfError"]

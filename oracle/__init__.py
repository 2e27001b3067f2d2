"""ctypes bindings of the C oracle (``oracle/*.c``): the FP64 restatement of the reference's
Chorin-projection path.  Test infrastructure only — imported by ``tests/``, by
``__graft_entry__.smoke()`` as the checker, and by ``bench.py``'s CPU-baseline leg; the product
package never imports it.

``reference()`` additionally loads ``oracle/_ref/libnsfref.so`` (the reference's own C++ built
from its sources by ``oracle/Makefile.ref``) when it has been built on this machine.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

i32p = C.POINTER(C.c_int)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)


class CsrS(C.Structure):
    _fields_ = [("rows", C.c_int), ("cols", C.c_int), ("nnz", C.c_int),
                ("rowStart", i32p), ("col", i32p), ("val", f64p)]


class MeshS(C.Structure):
    _fields_ = [("numCorner", C.c_int), ("numTri", C.c_int), ("numBorder", C.c_int), ("numGroups", C.c_int),
                ("cornerXY", f32p), ("tri", i32p), ("border", i32p), ("groups", C.POINTER(C.c_char_p)),
                ("numV", C.c_int), ("numP", C.c_int), ("vXY", f32p), ("vElem", i32p), ("vBorder", i32p),
                ("pElem", i32p), ("pBorder", i32p), ("affine", f32p)]


class ContextS(C.Structure):
    _fields_ = [("N", C.c_int), ("P", C.c_int), ("nDir", C.c_int), ("dirIds", i32p), ("dirVx", f64p),
                ("nDirP", C.c_int), ("dirPIds", i32p), ("nIntV", C.c_int), ("nIntP", C.c_int),
                ("intV", i32p), ("intP", i32p),
                ("M", CsrS), ("K", CsrS), ("Kp", CsrS), ("Kpi", CsrS), ("D", CsrS), ("G", CsrS), ("I", CsrS)]


class ColoringS(C.Structure):
    _fields_ = [("n", C.c_int), ("nColors", C.c_int), ("perm", i32p), ("partStart", i32p), ("slOrder", i32p)]


class ChorinCfgS(C.Structure):
    _fields_ = [("nu", C.c_double), ("tau", C.c_double), ("velMethod", C.c_int), ("velMaxIters", C.c_int),
                ("velTol", C.c_double), ("presMaxIters", C.c_int), ("presTol", C.c_double), ("presGuess", C.c_int),
                ("presBasis", C.c_int)]


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with make (plain C)."""
    out = subprocess.run(["make", "-C", HERE, "-s"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "_build", "liboracle.so")


_LIB_MT = None


def build_mt() -> bool:
    """Compile liboracle_mt.so (OpenMP); False if this toolchain cannot."""
    out = subprocess.run(["make", "-C", HERE, "-s", "mt"], capture_output=True, text=True)
    return out.returncode == 0


def lib_mt():
    """The OpenMP build of the oracle (the timed CPU baseline on all host cores), or None."""
    global _LIB_MT
    if _LIB_MT is None:
        path = os.path.join(HERE, "_build", "liboracle_mt.so")
        if not os.path.exists(path) and not build_mt():
            return None
        _LIB_MT = _configure(C.CDLL(path))
    return _LIB_MT


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            build()
        _LIB = _configure(C.CDLL(path))
    return _LIB


def _configure(L):
    if True:
        L.orc_last_error.restype = C.c_char_p
        L.orc_mesh_load.restype = C.POINTER(MeshS)
        L.orc_mesh_load.argtypes = [C.c_char_p]
        L.orc_mesh_free.argtypes = [C.POINTER(MeshS)]
        L.orc_group_id.argtypes = [C.POINTER(MeshS), C.c_char_p]
        L.orc_channel_bcs.argtypes = [C.POINTER(MeshS), C.c_float, C.POINTER(ContextS)]
        L.orc_assemble.argtypes = [C.POINTER(MeshS), C.POINTER(ContextS), C.c_int]
        L.orc_local_matrices.argtypes = [C.POINTER(MeshS), C.c_int, f64p]
        L.orc_context_free.argtypes = [C.POINTER(ContextS)]
        L.orc_csr_free.argtypes = [C.POINTER(CsrS)]
        L.orc_spmv.argtypes = [C.POINTER(CsrS), f64p, f64p]
        L.orc_cheb_iters.argtypes = [C.POINTER(CsrS), C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_cheb_solve.argtypes = [C.POINTER(CsrS), f64p, f64p, C.c_double, C.c_double, C.c_int, C.c_double,
                                     f64p]
        L.orc_spmm2.argtypes = [C.POINTER(CsrS), f64p, f64p, f64p]
        L.orc_slice.argtypes = [C.POINTER(CsrS), C.c_int, i32p, C.c_int, i32p, C.POINTER(CsrS)]
        L.orc_coloring_build.argtypes = [C.POINTER(CsrS), C.POINTER(ColoringS)]
        L.orc_coloring_free.argtypes = [C.POINTER(ColoringS)]
        L.orc_gs_solve.argtypes = [C.POINTER(CsrS), C.POINTER(ColoringS), C.c_int, f64p, f64p, C.c_int,
                                   C.c_double, C.c_int, f64p, i32p]
        L.orc_pcg.argtypes = [C.POINTER(CsrS), C.POINTER(ColoringS), C.c_int, f64p, f64p, C.c_int, C.c_double,
                              i32p, f64p]
        L.orc_sgs_apply.argtypes = [C.POINTER(CsrS), C.POINTER(ColoringS), f64p, f64p]
        L.orc_chorin_create.restype = C.c_void_p
        L.orc_chorin_create.argtypes = [C.POINTER(ContextS), C.POINTER(ChorinCfgS)]
        L.orc_chorin_free.argtypes = [C.c_void_p]
        L.orc_chorin_get.argtypes = [C.c_void_p, f64p, f64p]
        L.orc_chorin_set.argtypes = [C.c_void_p, f64p, f64p]
        L.orc_chorin_step.argtypes = [C.c_void_p, f64p]
        L.orc_fastconv.argtypes = [C.POINTER(ContextS), C.c_double, f64p, f64p]
        L.orc_forces.argtypes = [C.POINTER(MeshS), C.c_int, f64p, f64p, C.c_double, f64p]
        L.orc_chorin_set_dirichlet.argtypes = [C.c_void_p, f64p]
        L.orc_forces_weights.argtypes = [C.POINTER(MeshS), C.c_int, f64p, f64p, f64p]
        L.orc_adjoint_run.argtypes = [C.POINTER(ContextS), C.POINTER(MeshS), C.c_int, C.POINTER(ChorinCfgS), f64p,
                                      f64p, f64p, C.c_int, f64p, f64p, C.c_double, f64p, f64p, f64p]
    return L


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Csr:
    """Host CSR copy: rows, cols, rowStart (int32), col (int32), val (float64)."""

    def __init__(self, rows, cols, rowStart, col, val=None):
        self.rows, self.cols = int(rows), int(cols)
        self.rowStart = np.ascontiguousarray(rowStart, dtype=np.int32)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.val = None if val is None else np.ascontiguousarray(val, dtype=np.float64)

    @property
    def nnz(self):
        return int(self.col.shape[0])

    @staticmethod
    def from_struct(s: CsrS) -> "Csr":
        val = _arr(s.val, s.nnz, np.float64) if bool(s.val) else None
        return Csr(s.rows, s.cols, _arr(s.rowStart, s.rows + 1, np.int32), _arr(s.col, s.nnz, np.int32), val)

    def struct(self) -> CsrS:
        s = CsrS()
        s.rows, s.cols, s.nnz = self.rows, self.cols, self.nnz
        s.rowStart = _ptr(self.rowStart, C.c_int)
        s.col = _ptr(self.col, C.c_int)
        if self.val is None:
            self.val = np.zeros(self.nnz, dtype=np.float64)
        s.val = _ptr(self.val, C.c_double)
        return s

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rowStart), shape=(self.rows, self.cols))


class Mesh:
    """Oracle mesh: corner mesh, P2 velocity numbering and P1 pressure numbering."""

    def __init__(self, path: str):
        L = lib()
        p = L.orc_mesh_load(path.encode())
        if not p:
            raise RuntimeError("oracle mesh load failed: " + L.orc_last_error().decode())
        self._p = p
        m = p.contents
        self.num_corner, self.num_tri, self.num_border = m.numCorner, m.numTri, m.numBorder
        self.groups = [m.groups[i].decode() for i in range(m.numGroups)]
        self.corner_xy = _arr(m.cornerXY, 2 * m.numCorner, np.float32).reshape(-1, 2)
        self.tri = _arr(m.tri, 3 * m.numTri, np.int32).reshape(-1, 3)
        self.border = _arr(m.border, 3 * m.numBorder, np.int32).reshape(-1, 3)
        self.N, self.P = m.numV, m.numP
        self.v_xy = _arr(m.vXY, 2 * m.numV, np.float32).reshape(-1, 2)
        self.v_elem = _arr(m.vElem, 6 * m.numTri, np.int32).reshape(-1, 6)
        self.v_border = _arr(m.vBorder, 6 * m.numBorder, np.int32).reshape(-1, 6)
        self.p_elem = _arr(m.pElem, 3 * m.numTri, np.int32).reshape(-1, 3)
        self.p_border = _arr(m.pBorder, 5 * m.numBorder, np.int32).reshape(-1, 5)
        self.affine = _arr(m.affine, 6 * m.numTri, np.float32).reshape(-1, 6)

    LOCAL_SHAPES = (("mass", (6, 6)), ("stiff", (6, 6)), ("stiffP", (3, 3)), ("divX", (3, 6)), ("divY", (3, 6)),
                    ("gradX", (6, 3)), ("gradY", (6, 3)), ("conv", (12, 6, 6)))

    def local_matrices(self, e: int) -> dict:
        """FP64 local matrices of element e (orc_local_matrices), keyed as the reference harness's."""
        out = np.zeros(585)
        lib().orc_local_matrices(self._p, int(e), _ptr(out, C.c_double))
        res, o = {}, 0
        for k, shp in self.LOCAL_SHAPES:
            n = int(np.prod(shp))
            res[k] = out[o:o + n].reshape(shp)
            o += n
        return res

    def __del__(self):
        try:
            lib().orc_mesh_free(self._p)
        except Exception:
            pass


class Context:
    """Channel-problem context: Dirichlet/internal lists and the assembled FP64 matrices."""

    NAMES = ("M", "K", "Kp", "Kpi", "D", "G", "I")

    def __init__(self, mesh: Mesh, peak_velocity: float, with_convection: bool = True):
        L = lib()
        self._s = ContextS()
        if L.orc_channel_bcs(mesh._p, C.c_float(peak_velocity), C.byref(self._s)) != 0:
            raise RuntimeError(L.orc_last_error().decode())
        L.orc_assemble(mesh._p, C.byref(self._s), int(with_convection))
        s = self._s
        self.N, self.P = s.N, s.P
        self.dir_ids = _arr(s.dirIds, s.nDir, np.int32)
        self.dir_vx = _arr(s.dirVx, s.nDir, np.float64)
        self.dir_p_ids = _arr(s.dirPIds, s.nDirP, np.int32)
        self.int_v = _arr(s.intV, s.nIntV, np.int32)
        self.int_p = _arr(s.intP, s.nIntP, np.int32)
        for name in self.NAMES:
            cs = getattr(s, name)
            setattr(self, name, Csr.from_struct(cs) if cs.rows > 0 else None)

    def __del__(self):
        try:
            lib().orc_context_free(C.byref(self._s))
        except Exception:
            pass


def coloring(a: Csr):
    """(perm, partStart, slOrder) of the smallest-last + greedy coloring."""
    L = lib()
    s = a.struct()
    c = ColoringS()
    L.orc_coloring_build(C.byref(s), C.byref(c))
    out = (_arr(c.perm, c.n, np.int32), _arr(c.partStart, c.nColors + 1, np.int32), _arr(c.slOrder, c.n, np.int32))
    L.orc_coloring_free(C.byref(c))
    return out


def _col_struct(perm, part):
    c = ColoringS()
    c.n = len(perm)
    c.nColors = len(part) - 1
    c.perm = _ptr(perm, C.c_int)
    c.partStart = _ptr(part, C.c_int)
    c.slOrder = _ptr(perm, C.c_int)
    return c


def slice_csr(a: Csr, rows, cols) -> Csr:
    L = lib()
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    s = a.struct()
    o = CsrS()
    L.orc_slice(C.byref(s), len(rows), _ptr(rows, C.c_int), len(cols), _ptr(cols, C.c_int), C.byref(o))
    r = Csr.from_struct(o)
    L.orc_csr_free(C.byref(o))
    return r


def spmv(a: Csr, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.rows, dtype=np.float64)
    s = a.struct()
    lib().orc_spmv(C.byref(s), _ptr(x, C.c_double), _ptr(y, C.c_double))
    return y


# spectral bounds of D^-1 M for the P2 mass matrix (oracle.h ORC_MASS_SPEC_LO / _HI)
MASS_SPEC_LO, MASS_SPEC_HI = 0.39237, 2.05982


def cheb_iters(a: Csr, rel_tol, max_iters=100000, lo=MASS_SPEC_LO, hi=MASS_SPEC_HI) -> int:
    """A priori Chebyshev-Jacobi iteration count for ||r|| <= rel_tol ||b|| (orc_cheb_iters)."""
    s = a.struct()
    return int(lib().orc_cheb_iters(C.byref(s), lo, hi, rel_tol, max_iters))


def cheb_solve(a: Csr, b, iters, rel_tol, lo=MASS_SPEC_LO, hi=MASS_SPEC_HI):
    """x from `iters` Chebyshev-Jacobi iterations from 0; returns (x, status, relative residual)."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(a.rows, dtype=np.float64)
    rr = np.zeros(1, dtype=np.float64)
    s = a.struct()
    st = lib().orc_cheb_solve(C.byref(s), _ptr(b, C.c_double), _ptr(x, C.c_double), lo, hi, iters, rel_tol,
                              _ptr(rr, C.c_double))
    return x, int(st), float(rr[0])


def spmm2(a: Csr, vals, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    y = np.zeros(2 * a.rows, dtype=np.float64)
    s = a.struct()
    lib().orc_spmm2(C.byref(s), _ptr(vals, C.c_double), _ptr(x, C.c_double), _ptr(y, C.c_double))
    return y


def gs_solve(a: Csr, col, num_ch, b, x0, max_iters, target_rms, check_interval=1):
    perm, part = col[0], col[1]
    x = np.array(x0, dtype=np.float64, copy=True)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rms = np.zeros(num_ch, dtype=np.float64)
    it = C.c_int(0)
    s = a.struct()
    cs = _col_struct(perm, part)
    rc = lib().orc_gs_solve(C.byref(s), C.byref(cs), num_ch, _ptr(b, C.c_double), _ptr(x, C.c_double), max_iters,
                            target_rms, check_interval, _ptr(rms, C.c_double), C.byref(it))
    if rc != 0:
        raise RuntimeError("oracle GS failed (zero or missing diagonal)")
    return x, rms, it.value


def pcg(a: Csr, col, b, x0, max_iters, rel_tol, precond=1):
    perm, part = col[0], col[1]
    x = np.array(x0, dtype=np.float64, copy=True)
    b = np.ascontiguousarray(b, dtype=np.float64)
    it = C.c_int(0)
    rr = C.c_double(0)
    s = a.struct()
    cs = _col_struct(perm, part)
    st = lib().orc_pcg(C.byref(s), C.byref(cs), precond, _ptr(b, C.c_double), _ptr(x, C.c_double), max_iters,
                       rel_tol, C.byref(it), C.byref(rr))
    return x, st, it.value, rr.value


def sgs_apply(a: Csr, col, r):
    perm, part = col[0], col[1]
    r = np.ascontiguousarray(r, dtype=np.float64)
    z = np.zeros_like(r)
    s = a.struct()
    cs = _col_struct(perm, part)
    lib().orc_sgs_apply(C.byref(s), C.byref(cs), _ptr(r, C.c_double), _ptr(z, C.c_double))
    return z


def fastconv(ctx: Context, nu: float, u) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros(ctx.K.nnz, dtype=np.float64)
    lib().orc_fastconv(C.byref(ctx._s), nu, _ptr(u, C.c_double), _ptr(out, C.c_double))
    return out


def forces(mesh: Mesh, u, p, nu: float, group: str = "Circle") -> np.ndarray:
    """(F_x, F_y) = integral over the border group of (-p n + nu du/dn), n into the fluid."""
    L = lib()
    gid = L.orc_group_id(mesh._p, group.encode())
    if gid < 0:
        raise ValueError(f"no border group {group!r}")
    u = np.ascontiguousarray(u, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros(2, dtype=np.float64)
    L.orc_forces(mesh._p, gid, _ptr(u, C.c_double), _ptr(p, C.c_double), nu, _ptr(out, C.c_double))
    return out


class Chorin:
    """FP64 Chorin stepper of the oracle.  vel_method 0 = multicolor GS (RMS target),
    1 = CG + multicolor SGS, 2 = CG + Jacobi, 3 = Chebyshev-Jacobi, 4 = Chebyshev-Jacobi warm-started from
    the previous step (relative tolerance).  mt: run on the OpenMP build
    (all host threads, OMP_NUM_THREADS); self.threads says what ran (1 if that build is missing)."""

    def __init__(self, ctx: Context, nu, tau, vel_method=1, vel_max_iters=200, vel_tol=1e-10,
                 pres_max_iters=2000, pres_tol=1e-10, mt=False, pres_guess=0, pres_basis=0):
        self.ctx = ctx
        self._L = lib_mt() if mt else None
        self.threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)) if self._L else 1
        if self._L is None:
            self._L = lib()
        cfg = ChorinCfgS(nu, tau, vel_method, vel_max_iters, vel_tol, pres_max_iters, pres_tol, pres_guess,
                         pres_basis)
        self._h = self._L.orc_chorin_create(C.byref(ctx._s), C.byref(cfg))

    def step(self):
        st = np.zeros(6, dtype=np.float64)
        rc = self._L.orc_chorin_step(self._h, _ptr(st, C.c_double))
        if rc != 0:
            raise RuntimeError(f"oracle Chorin step failed with status {rc}")
        return st

    def state(self):
        u = np.zeros(2 * self.ctx.N, dtype=np.float64)
        p = np.zeros(self.ctx.P, dtype=np.float64)
        self._L.orc_chorin_get(self._h, _ptr(u, C.c_double), _ptr(p, C.c_double))
        return u, p

    def set_state(self, u, p):
        u = np.ascontiguousarray(u, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        self._L.orc_chorin_set(self._h, _ptr(u, C.c_double), _ptr(p, C.c_double))

    def set_dirichlet(self, dir_vx):
        """x values of the Dirichlet velocity nodes (ctx.dir_ids order), imposed on the state too."""
        d = np.ascontiguousarray(dir_vx, dtype=np.float64)
        if d.shape != (len(self.ctx.dir_ids),):
            raise ValueError("one value per Dirichlet node")
        self._L.orc_chorin_set_dirichlet(self._h, _ptr(d, C.c_double))

    def __del__(self):
        try:
            self._L.orc_chorin_free(self._h)
        except Exception:
            pass


def forces_weights(mesh: Mesh, group: str = "Circle"):
    """(wV, wPx, wPy): F_x = nu wV.u_x + wPx.p and F_y = nu wV.u_y + wPy.p."""
    L = lib()
    gid = L.orc_group_id(mesh._p, group.encode())
    if gid < 0:
        raise ValueError(f"no border group {group!r}")
    wV = np.zeros(mesh.N, dtype=np.float64)
    wPx = np.zeros(mesh.P, dtype=np.float64)
    wPy = np.zeros(mesh.P, dtype=np.float64)
    L.orc_forces_weights(mesh._p, gid, _ptr(wV, C.c_double), _ptr(wPx, C.c_double), _ptr(wPy, C.c_double))
    return wV, wPx, wPy


def adjoint_run(ctx: Context, mesh: Mesh, nu, tau, n_steps, w_drag, w_lift=None, dir_vx=None, u0=None, p0=None,
                vel_method=1, vel_max_iters=100000, vel_tol=1e-14, pres_max_iters=100000, pres_tol=1e-14,
                solve_tol=1e-14, group: str = "Circle", mt=False):
    """FP64 forward + discrete-adjoint sweep of the oracle (orc_adjoint_run); mt: the OpenMP build
    (falls back to the single-thread build if it is missing).

    Returns (J, dJ/dnu, dJ/d dirVx [nDir], dJ/du0 [2N])."""
    L = (lib_mt() if mt else None) or lib()
    gid = L.orc_group_id(mesh._p, group.encode())
    if gid < 0:
        raise ValueError(f"no border group {group!r}")
    cfg = ChorinCfgS(nu, tau, vel_method, vel_max_iters, vel_tol, pres_max_iters, pres_tol)
    d = np.ascontiguousarray(ctx.dir_vx if dir_vx is None else dir_vx, dtype=np.float64)
    wd = np.ascontiguousarray(np.broadcast_to(np.asarray(w_drag, dtype=np.float64), (n_steps,)))
    wl = np.zeros(n_steps) if w_lift is None else np.asarray(w_lift, dtype=np.float64)
    wl = np.ascontiguousarray(np.broadcast_to(wl, (n_steps,)))
    uu = None if u0 is None else np.ascontiguousarray(u0, dtype=np.float64)
    pp = None if p0 is None else np.ascontiguousarray(p0, dtype=np.float64)
    out = np.zeros(2)
    gdir = np.zeros(len(ctx.dir_ids) + 1)
    gu = np.zeros(2 * ctx.N)
    rc = L.orc_adjoint_run(C.byref(ctx._s), mesh._p, gid, C.byref(cfg), _ptr(d, C.c_double),
                           None if uu is None else _ptr(uu, C.c_double),
                           None if pp is None else _ptr(pp, C.c_double), int(n_steps), _ptr(wd, C.c_double),
                           _ptr(wl, C.c_double), solve_tol, _ptr(out, C.c_double), _ptr(gdir, C.c_double),
                           _ptr(gu, C.c_double))
    if rc != 0:
        raise RuntimeError(f"oracle adjoint failed with status {rc}")
    return float(out[0]), float(out[1]), gdir[:len(ctx.dir_ids)].copy(), gu


def forward_functional(ctx: Context, mesh: Mesh, nu, tau, n_steps, w_drag, w_lift=None, dir_vx=None,
                       vel_tol=1e-14, pres_tol=1e-14, group: str = "Circle"):
    """J of adjoint_run from a forward run alone (for finite differences)."""
    s = Chorin(ctx, nu, tau, vel_method=1, vel_max_iters=100000, vel_tol=vel_tol, pres_max_iters=100000,
               pres_tol=pres_tol)
    if dir_vx is not None:
        s.set_dirichlet(dir_vx)
    wd = np.broadcast_to(np.asarray(w_drag, dtype=np.float64), (n_steps,))
    wl = np.broadcast_to(np.asarray(0.0 if w_lift is None else w_lift, dtype=np.float64), (n_steps,))
    J = 0.0
    for n in range(n_steps):
        s.step()
        if wd[n] != 0 or wl[n] != 0:
            u, p = s.state()
            f = forces(mesh, u, p, nu, group)
            J += wd[n] * f[0] + wl[n] * f[1]
    return J


# ---------------------------------------------------------------- reference build (oracle/_ref)

def reference_path() -> str:
    return os.path.join(HERE, "_ref", "libnsfref.so")


def reference_root() -> str:
    """The reference's ``cpp`` tree: ``$NSFEM_REFERENCE_CPP`` if set, else the default ``REF`` of the
    build recipe ``oracle/Makefile.ref`` (the one place that names where the tree lies)."""
    env = os.environ.get("NSFEM_REFERENCE_CPP")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile.ref")) as f:
        for line in f:
            if line.startswith("REF ?="):
                return line.split("?=", 1)[1].strip()
    return ""


def build_reference(ref_root: str | None = None) -> bool:
    """Build oracle/_ref/libnsfref.so from the reference sources if they are present."""
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(ref_root):
        return False
    out = subprocess.run(["make", "-C", HERE, "-f", "Makefile.ref", "-s", "-j8", f"REF={ref_root}"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference harness build failed:\n" + out.stdout + out.stderr)
    return True


def reference():
    """The reference-code harness, or None if it has not been built on this machine."""
    global _REF
    if _REF is None:
        p = reference_path()
        if not os.path.exists(p):
            return None
        try:
            R = C.CDLL(p)
        except OSError:
            return None
        R.ref_last_error.restype = C.c_char_p
        R.ref_mesh_load.restype = C.c_void_p
        R.ref_mesh_load.argtypes = [C.c_char_p]
        R.ref_mesh_free.argtypes = [C.c_void_p]
        R.ref_mesh_counts.argtypes = [C.c_void_p, i32p]
        R.ref_mesh_group.restype = C.c_char_p
        R.ref_mesh_group.argtypes = [C.c_void_p, C.c_int]
        R.ref_mesh_elements.argtypes = [C.c_void_p, C.c_int, i32p]
        R.ref_mesh_nodes.argtypes = [C.c_void_p, C.c_int, f32p]
        R.ref_mesh_border.argtypes = [C.c_void_p, C.c_int, i32p]
        R.ref_dirichlet.argtypes = [C.c_void_p, C.c_float, i32p, i32p, f32p, i32p, i32p, i32p]
        R.ref_prototype.restype = C.c_void_p
        R.ref_prototype.argtypes = [C.c_void_p, C.c_int]
        R.ref_csr_wrap.restype = C.c_void_p
        R.ref_csr_wrap.argtypes = [C.c_int, C.c_int, C.c_int, i32p, i32p, f32p]
        R.ref_csr_free.argtypes = [C.c_void_p]
        R.ref_csr_dims.argtypes = [C.c_void_p, i32p]
        R.ref_csr_arrays.argtypes = [C.c_void_p, i32p, i32p, f32p]
        R.ref_csr_slice.restype = C.c_void_p
        R.ref_csr_slice.argtypes = [C.c_void_p, C.c_int, i32p, C.c_int, i32p]
        R.ref_coloring.restype = C.c_int
        R.ref_coloring.argtypes = [C.c_void_p, i32p, i32p, i32p]
        R.ref_gs2ch_double.argtypes = [C.c_int, i32p, i32p, f64p, f64p, f64p, C.c_int, C.c_double, f64p]
        R.ref_rmult_double.argtypes = [C.c_int, C.c_int, i32p, i32p, f64p, f64p, f64p]
        R.ref_assembled.restype = C.c_int
        R.ref_assembled.argtypes = [C.c_void_p, C.c_int, i32p, i32p, i32p, f32p]
        R.ref_local_matrices.restype = C.c_int
        R.ref_local_matrices.argtypes = [C.c_void_p, C.c_int] + [f32p] * 8
        R.ref_fastconv_values.restype = C.c_int
        R.ref_fastconv_values.argtypes = [C.c_void_p, f32p]
        R.ref_io_write_csr.restype = C.c_int
        R.ref_io_write_csr.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, i32p, i32p, f64p]
        R.ref_io_read_csr.restype = C.c_int
        R.ref_io_read_csr.argtypes = [C.c_char_p, C.c_int, i32p, i32p, i32p, f64p]
        R.ref_io_write_vec.restype = C.c_int
        R.ref_io_write_vec.argtypes = [C.c_char_p, C.c_int, C.c_int, f64p]
        R.ref_io_read_vec.restype = C.c_int
        R.ref_io_read_vec.argtypes = [C.c_char_p, C.c_int, i32p, f64p]
        _REF = R
    return _REF


REF_ASSEMBLED = ("M", "K", "Kp", "D", "G")  # ref_assembled's `which` order


def reference_assembled(R, h, name: str) -> Csr:
    """The reference's assembled FP32 operator `name` (M, K, Kp, D, G) for the harness mesh h, or
    "I" for the FastConvection integration matrix (values from the reference's integrator)."""
    if name == "I":
        ph = R.ref_prototype(h, 4)
        dims = (C.c_int * 3)()
        R.ref_csr_dims(ph, dims)
        rs = np.zeros(dims[0] + 1, np.int32)
        cl = np.zeros(dims[2], np.int32)
        R.ref_csr_arrays(ph, _ptr(rs, C.c_int), _ptr(cl, C.c_int), None)
        R.ref_csr_free(ph)
        val = np.zeros(dims[2], np.float32)
        if R.ref_fastconv_values(h, _ptr(val, C.c_float)) != 0:
            raise RuntimeError(R.ref_last_error().decode())
        return Csr(dims[0], dims[1], rs, cl, val)
    w = REF_ASSEMBLED.index(name)
    dims = (C.c_int * 3)()
    if R.ref_assembled(h, w, dims, None, None, None) != 0:
        raise RuntimeError(R.ref_last_error().decode())
    rs = np.zeros(dims[0] + 1, np.int32)
    cl = np.zeros(dims[2], np.int32)
    val = np.zeros(dims[2], np.float32)
    R.ref_assembled(h, w, dims, _ptr(rs, C.c_int), _ptr(cl, C.c_int), _ptr(val, C.c_float))
    return Csr(dims[0], dims[1], rs, cl, val)


def reference_local_matrices(R, h, e: int) -> dict:
    """The reference integrator's FP32 local matrices of element e (see ref_local_matrices)."""
    shapes = {"mass": (6, 6), "stiff": (6, 6), "stiffP": (3, 3), "divX": (3, 6), "divY": (3, 6),
              "gradX": (6, 3), "gradY": (6, 3), "conv": (12, 6, 6)}
    out = {k: np.zeros(v, np.float32) for k, v in shapes.items()}
    if R.ref_local_matrices(h, int(e), *[_ptr(out[k], C.c_float) for k in shapes]) != 0:
        raise RuntimeError(R.ref_last_error().decode())
    return out

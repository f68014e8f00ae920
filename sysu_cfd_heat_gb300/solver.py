"""Python mirror of the reference's solver interface over the C ABI.

``NavierStokesSolver`` keeps the method names of the reference class (navier.h:73-123):
``NSSolve``, ``CalculateVelocity``, ``CalculatePressure``, ``UpdateTurKEpsilon``,
``UpdateEnergy``, the ``Residual`` monitor, and field access by member name; the solid
module of a conjugate case is reachable as ``physicalModule["3dHeatConduction"]`` with its
``solve()`` (HeatConductionSolver.h:37).  Everything runs on the GPU through
libsysucfd.so; errors the reference would ``exit()`` on raise ``SysuError``.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from ._lib import SysuError, _dptr, check, lib

SLOTS = ("mom", "p", "k", "eps", "T", "solid_T")


class HeatConductionSolver:
    """Solid conduction module of a conjugate case (HeatConductionSolver.cpp)."""

    def __init__(self, parent: "NavierStokesSolver"):
        self._p = parent

    def solve(self) -> None:
        check(lib().sysu_solver_heat_conduction(self._p._h))

    @property
    def Tn(self) -> np.ndarray:
        return self._p.get("solid_T")


class NavierStokesSolver:
    def __init__(self, paramfile: str, options: Optional[Dict[str, float]] = None):
        self._h = C.c_void_p()
        check(lib().sysu_solver_create(paramfile.encode(), C.byref(self._h)))
        for k, v in (options or {}).items():
            self.set_option(k, v)
        self.physicalModule = {}
        if self.info()["solid_Ncel"] > 0:
            self.physicalModule["3dHeatConduction"] = HeatConductionSolver(self)

    @classmethod
    def _borrow(cls, handle: int) -> "NavierStokesSolver":
        """A view of a solver owned elsewhere (a case of a batch): close() does not free it."""
        self = cls.__new__(cls)
        self._h = C.c_void_p(handle)
        self._borrowed = True
        self.physicalModule = {}
        if self.info()["solid_Ncel"] > 0:
            self.physicalModule["3dHeatConduction"] = HeatConductionSolver(self)
        return self

    def close(self) -> None:
        if self._h and not getattr(self, "_borrowed", False):
            lib().sysu_solver_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- configuration -------------------------------------------------------------
    def set_option(self, key: str, value: float) -> None:
        check(lib().sysu_solver_set_option(self._h, key.encode(), float(value)))

    def get_option(self, key: str) -> float:
        v = C.c_double()
        check(lib().sysu_solver_get_option(self._h, key.encode(), C.byref(v)))
        return v.value

    def info(self) -> dict:
        out = (C.c_long * 6)()
        check(lib().sysu_solver_info(self._h, out, 6))
        return dict(zip(["Ncel", "Nfac", "Nbnd", "solid_Ncel", "nnz_stored", "nnz"], list(out)))

    # -- the reference's driver methods -----------------------------------------------
    def NSSolve(self) -> int:
        done = C.c_int()
        check(lib().sysu_solver_nssolve(self._h, C.byref(done)))
        return done.value

    def Output(self, directory: str = None) -> None:
        """NavierStokesSolver::Output: tec/res####.dat (numbered from 0) in `directory`
        (default: the directory of param.in), text identical to the reference's."""
        check(lib().sysu_solver_output(self._h, directory.encode() if directory else None))

    def VolumnAverage(self, t: float, out_iter: int, directory: str = None) -> None:
        """NavierStokesSolver::VolumnAverage: one line of tot.dat (header when new)."""
        check(lib().sysu_solver_volume_average(self._h, directory.encode() if directory else None, float(t),
                                               int(out_iter)))

    def iterate(self, n: int) -> int:
        """Run up to n steady outer iterations (stops at the steady convergence test)."""
        done = C.c_int()
        check(lib().sysu_solver_iterate(self._h, int(n), C.byref(done)))
        return done.value

    def CalculateVelocity(self) -> None:
        check(lib().sysu_solver_calculate_velocity(self._h))

    def CalculatePressure(self) -> None:
        check(lib().sysu_solver_calculate_pressure(self._h))

    def UpdateTurKEpsilon(self) -> None:
        check(lib().sysu_solver_update_turkeps(self._h))

    def SaveTransientOldData(self) -> None:
        check(lib().sysu_solver_save_transient_old_data(self._h))

    def UpdateEnergy(self) -> None:
        check(lib().sysu_solver_update_energy(self._h))

    def check(self) -> None:
        """Read the residual monitor and apply the reference's convergence checks."""
        check(lib().sysu_solver_check(self._h))

    def sync(self) -> None:
        check(lib().sysu_solver_sync(self._h))

    def reset(self) -> None:
        """Back to the state right after creation (InitFlowField)."""
        check(lib().sysu_solver_reset(self._h))

    def timer_start(self) -> None:
        check(lib().sysu_solver_timer_start(self._h))

    def timer_stop(self) -> float:
        """Device time (ms) on the solver's stream since timer_start()."""
        ms = C.c_double()
        check(lib().sysu_solver_timer_stop(self._h, C.byref(ms)))
        return ms.value

    @property
    def Residual(self) -> np.ndarray:
        out = np.zeros(10)
        check(lib().sysu_solver_residuals(self._h, _dptr(out)))
        return out

    def solve_stats(self) -> Dict[str, dict]:
        it = (C.c_int * 18)()
        rs = np.zeros(18)
        stt = (C.c_int * 18)()
        check(lib().sysu_solver_solve_stats(self._h, it, _dptr(rs), stt))
        out = {}
        for k, name in enumerate(SLOTS):
            out[name] = {"iters": list(it[3 * k:3 * k + 3]), "res": rs[3 * k:3 * k + 3].tolist(),
                         "status": list(stt[3 * k:3 * k + 3])}
        return out

    def timing(self) -> tuple:
        p = C.c_double()
        m = C.c_double()
        check(lib().sysu_solver_timing(self._h, C.byref(p), C.byref(m)))
        return p.value, m.value

    def spmv_timing(self, which: str = "p", fp32: bool = False, reps: int = 10, steady: bool = False) -> float:
        """Mean device ms of one standalone y = A x on an assembled matrix: L2 flushed
        before each product, or (steady) products back to back alternating between
        two full copies of the operands."""
        ms = C.c_double()
        fn = lib().sysu_solver_spmv_timing_steady if steady else lib().sysu_solver_spmv_timing
        check(fn(self._h, which.encode(), int(fp32), int(reps), C.byref(ms)))
        return ms.value

    def cg_phases(self) -> np.ndarray:
        """%globaltimer stamps (ns) of the last CG solve, shape (64, 4): iteration
        start, after the direction update, after the product, after the update
        (option profile_phases)."""
        ts = np.zeros(256, np.uint64)
        check(lib().sysu_solver_cg_phases(self._h, ts.ctypes.data, 256))
        return ts.reshape(64, 4)

    # -- fields ----------------------------------------------------------------------
    def field_size(self, name: str) -> int:
        n = lib().sysu_solver_field_size(self._h, name.encode())
        if n < 0:
            raise KeyError(name)
        return n

    def get(self, name: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Field by the reference's member name; into `out` (contiguous float64,
        e.g. page-locked from _lib.pinned_empty) when given."""
        n = self.field_size(name)
        if out is None:
            out = np.empty(n, dtype=np.float64)
        elif out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
            raise ValueError(f"out must be a contiguous float64 array of {n} values")
        check(lib().sysu_solver_get_field(self._h, name.encode(), _dptr(out), n))
        return out

    def p_cycle(self, r, use_net: bool = True) -> np.ndarray:
        """One application of the p' multigrid cycle (option p.precond 4) as the
        last p' solve left it, z = M r."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros_like(r)
        check(lib().sysu_solver_p_cycle(self._h, _dptr(r), _dptr(z), 1 if use_net else 0))
        return z

    def p_network(self):
        """(level, parameters) of the p' network: level 0 the finest, >= 1 a
        coarse level of the multigrid cycle."""
        lvl = C.c_int()
        n = lib().sysu_gnn_num_params()
        prm = np.zeros(n, np.float32)
        check(lib().sysu_solver_p_network(self._h, C.byref(lvl), prm.ctypes.data_as(C.POINTER(C.c_float)), n))
        return lvl.value, prm

    def p_set_network(self, params) -> None:
        prm = np.ascontiguousarray(params, dtype=np.float32)
        check(lib().sysu_solver_p_set_network(self._h, prm.ctypes.data_as(C.POINTER(C.c_float)), len(prm)))

    def set(self, name: str, values) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        check(lib().sysu_solver_set_field(self._h, name.encode(), _dptr(a), a.size))

    def matrix(self, which: str):
        """Assembled matrix as (rowptr, col, val), diagonal first in each row."""
        L = lib()
        L.sysu_solver_matrix.restype = C.c_long
        L.sysu_solver_matrix.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]
        nnz = L.sysu_solver_matrix(self._h, which.encode(), None, None, None)
        if nnz < 0:
            raise KeyError(which)
        n = self.info()["solid_Ncel"] if which == "solid" else self.info()["Ncel"]
        rp = np.empty(n + 1, np.int32)
        cl = np.empty(nnz, np.int32)
        vl = np.empty(nnz, np.float64)
        got = L.sysu_solver_matrix(self._h, which.encode(), rp.ctypes.data, cl.ctypes.data, vl.ctypes.data)
        if got != nnz:
            raise SysuError(1, "matrix read-back failed")
        return rp, cl, vl


def csr_solve(rowptr, col, val, b, x0=None, method: str = "CG", precond: str = "Jacobi", maxit: int = 1000,
              eps: float = 1e-8, omega: float = 1.0):
    """GPU Krylov solve of a host CSR system; returns (x, iters, res, status)."""
    L = lib()
    fn = L.sysu_csr_solve
    fn.restype = C.c_int
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    fn.argtypes = [C.c_int, C.c_int, C.c_int, ip, ip, dp, dp, dp, C.c_int, C.c_double, C.c_double, ip, dp, ip]
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    n = len(rowptr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    it, rs, stt = C.c_int(), C.c_double(), C.c_int()
    if method == "CG-multigrid":
        precond = "multigrid"
    code = fn({"CG": 0, "BiCGSTAB": 1, "CG-mixed": 2, "GMRES": 3, "BiCGSTAB-mixed": 4, "CG-multigrid": 5}[method],
              {"none": 0, "Jacobi": 1, "SSOR": 2, "ILU": 3, "multigrid": 4}[precond], n,
              rowptr.ctypes.data_as(ip), col.ctypes.data_as(ip), _dptr(val), _dptr(b), _dptr(x), maxit, eps, omega,
              C.byref(it), C.byref(rs), C.byref(stt))
    if code != 0:
        L.sysu_csr_last_error.restype = C.c_char_p
        raise SysuError(code, L.sysu_csr_last_error().decode())
    return x, it.value, rs.value, stt.value


def csr_bicgstab3(rowptr, col, val, B, X0=None, mixed: bool = False, maxit: int = 500, eps: float = 1e-8,
                  omega: float = 1.0, inner_tol: float = 0.1):
    """Three right-hand sides B[c] of one CSR matrix (the momentum form) by BiCGSTAB +
    Jacobi: FP64, or (mixed) FP32 recurrences with FP64 residual replacement.
    Returns (X (3 x n), iters[3], res[3], status[3], refinements)."""
    L = lib()
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    n = len(rowptr) - 1
    B = [np.ascontiguousarray(B[c], np.float64) for c in range(3)]
    X = [np.zeros(n) if X0 is None else np.array(X0[c], dtype=np.float64) for c in range(3)]
    bp = (dp * 3)(*[_dptr(b) for b in B])
    xp = (dp * 3)(*[_dptr(x) for x in X])
    it, rs, stt, ref = (C.c_int * 3)(), (C.c_double * 3)(), (C.c_int * 3)(), C.c_int()
    code = L.sysu_csr_bicgstab3(n, rowptr.ctypes.data_as(ip), col.ctypes.data_as(ip), _dptr(val), bp, xp,
                                1 if mixed else 0, int(maxit), float(eps), float(omega), float(inner_tol), it, rs,
                                stt, C.byref(ref))
    if code != 0:
        L.sysu_csr_last_error.restype = C.c_char_p
        raise SysuError(code, L.sysu_csr_last_error().decode())
    return np.stack(X), list(it), list(rs), list(stt), ref.value


def csr_spmv_timing(rowptr, col, val, fp32: bool = False, reps: int = 10) -> float:
    """Mean device ms of one y = A x (L2 flushed before each) for a host CSR matrix."""
    L = lib()
    ip = C.POINTER(C.c_int)
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    ms = C.c_double()
    code = L.sysu_csr_spmv_timing(len(rowptr) - 1, rowptr.ctypes.data_as(ip), col.ctypes.data_as(ip), _dptr(val),
                                  1 if fp32 else 0, int(reps), C.byref(ms))
    if code != 0:
        L.sysu_csr_last_error.restype = C.c_char_p
        raise SysuError(code, L.sysu_csr_last_error().decode())
    return ms.value


def set_spmv_variant(variant: int) -> None:
    """Kernel form of the standalone SpMV (csr_spmv, spmv_timing), process-wide:
    0 one row per thread (default), 100 persistent ring with bulk copies."""
    if lib().sysu_set_spmv_variant(int(variant)) != 0:
        raise RuntimeError(lib().sysu_csr_last_error().decode())


def csr_spmv(rowptr, col, val, x):
    L = lib()
    fn = L.sysu_csr_spmv
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, ip, ip, dp, dp, dp]
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros(len(rowptr) - 1)
    code = fn(len(y), rowptr.ctypes.data_as(ip), col.ctypes.data_as(ip), _dptr(val), _dptr(x), _dptr(y))
    if code != 0:
        L.sysu_csr_last_error.restype = C.c_char_p
        raise SysuError(code, L.sysu_csr_last_error().decode())
    return y

"""ctypes binding of libsysucfd.so (the C ABI in include/sysu_cfd.h).

The library is loaded from the package directory only; if it is missing the import
fails loudly -- there is no CPU fallback for any solver entry point.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libsysucfd.so")

_lib = None


class SysuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with python -m sysu_cfd_heat_gb300.build")
        L = C.CDLL(LIB_PATH)
        vp, cp, ip, dp, lp = C.c_void_p, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_long)
        fp = C.POINTER(C.c_float)
        sig = {
            "sysu_last_error": (cp, []),
            "sysu_version": (C.c_int, []),
            "sysu_case_load": (C.c_int, [cp, C.POINTER(vp)]),
            "sysu_case_free": (None, [vp]),
            "sysu_case_info": (C.c_int, [vp, lp, C.c_int]),
            "sysu_case_array": (C.c_long, [vp, cp, vp, C.c_long]),
            "sysu_solver_create": (C.c_int, [cp, C.POINTER(vp)]),
            "sysu_solver_destroy": (None, [vp]),
            "sysu_solver_info": (C.c_int, [vp, lp, C.c_int]),
            "sysu_solver_set_option": (C.c_int, [vp, cp, C.c_double]),
            "sysu_solver_get_option": (C.c_int, [vp, cp, dp]),
            "sysu_solver_iterate": (C.c_int, [vp, C.c_int, ip]),
            "sysu_solver_nssolve": (C.c_int, [vp, ip]),
            "sysu_solver_calculate_velocity": (C.c_int, [vp]),
            "sysu_solver_calculate_pressure": (C.c_int, [vp]),
            "sysu_solver_update_turkeps": (C.c_int, [vp]),
            "sysu_solver_update_energy": (C.c_int, [vp]),
            "sysu_solver_heat_conduction": (C.c_int, [vp]),
            "sysu_solver_check": (C.c_int, [vp]),
            "sysu_solver_residuals": (C.c_int, [vp, dp]),
            "sysu_solver_solve_stats": (C.c_int, [vp, ip, dp, ip]),
            "sysu_solver_timing": (C.c_int, [vp, dp, dp]),
            "sysu_solver_field_size": (C.c_long, [vp, cp]),
            "sysu_solver_get_field": (C.c_int, [vp, cp, dp, C.c_long]),
            "sysu_solver_set_field": (C.c_int, [vp, cp, dp, C.c_long]),
            "sysu_solver_sync": (C.c_int, [vp]),
            "sysu_solver_p_cycle": (C.c_int, [vp, dp, dp, C.c_int]),
            "sysu_solver_p_network": (C.c_int, [vp, ip, C.POINTER(C.c_float), C.c_int]),
            "sysu_solver_p_set_network": (C.c_int, [vp, C.POINTER(C.c_float), C.c_int]),
            "sysu_solver_reset": (C.c_int, [vp]),
            "sysu_solver_timer_start": (C.c_int, [vp]),
            "sysu_solver_timer_stop": (C.c_int, [vp, dp]),
            "sysu_kernel_launches": (C.c_long, []),
            "sysu_solver_cg_phases": (C.c_int, [vp, vp, C.c_int]),
            "sysu_solver_spmv_timing": (C.c_int, [vp, cp, C.c_int, C.c_int, dp]),
            "sysu_solver_spmv_timing_steady": (C.c_int, [vp, cp, C.c_int, C.c_int, dp]),
            "sysu_solver_output": (C.c_int, [vp, cp]),
            "sysu_solver_save_transient_old_data": (C.c_int, [vp]),
            "sysu_solver_volume_average": (C.c_int, [vp, cp, C.c_double, C.c_int]),
            "sysu_solver_matrix": (C.c_long, [vp, cp, vp, vp, vp]),
            "sysu_csr_solve": (C.c_int, [C.c_int, C.c_int, C.c_int, ip, ip, dp, dp, dp, C.c_int, C.c_double,
                                         C.c_double, ip, dp, ip]),
            "sysu_csr_spmv": (C.c_int, [C.c_int, ip, ip, dp, dp, dp]),
            "sysu_set_spmv_variant": (C.c_int, [C.c_int]),
            "sysu_csr_spmv_timing": (C.c_int, [C.c_int, ip, ip, dp, C.c_int, C.c_int, dp]),
            "sysu_csr_last_error": (cp, []),
            "sysu_graph_loop_selftest": (C.c_int, [C.c_int, C.c_int, ip]),
            "sysu_csr_bicgstab_batched3": (C.c_int, [C.c_int, ip, ip, C.POINTER(dp), C.POINTER(dp), C.POINTER(dp),
                                                     C.c_int, C.c_double, ip, dp, ip]),
            "sysu_csr_bicgstab3": (C.c_int, [C.c_int, ip, ip, dp, C.POINTER(dp), C.POINTER(dp), C.c_int, C.c_int,
                                             C.c_double, C.c_double, C.c_double, ip, dp, ip, ip]),
            "sysu_setup_phases": (C.c_int, [dp]),
            "sysu_host_alloc": (vp, [C.c_size_t]),
            "sysu_host_free": (None, [vp]),
            "sysu_batch_create": (C.c_int, [C.c_int, C.POINTER(cp), C.POINTER(vp)]),
            "sysu_batch_free": (None, [vp]),
            "sysu_batch_size": (C.c_int, [vp]),
            "sysu_batch_case": (vp, [vp, C.c_int]),
            "sysu_batch_tune": (C.c_int, [vp, ip, C.c_int, ip, dp, dp, dp]),
            "sysu_batch_set_caps": (C.c_int, [vp, ip]),
            "sysu_batch_capture": (C.c_int, [vp]),
            "sysu_batch_replay": (C.c_int, [vp, C.c_int, dp]),
            "sysu_batch_check": (C.c_int, [vp]),
            "sysu_batch_run_sequential": (C.c_int, [vp, C.c_int, dp]),
            "sysu_gnn_num_params": (C.c_int, []),
            "sysu_gnn_create": (C.c_int, [C.c_int, ip, ip, dp, C.c_int, C.POINTER(vp)]),
            "sysu_gnn_free": (None, [vp]),
            "sysu_gnn_set_values": (C.c_int, [vp, ip, ip, dp]),
            "sysu_gnn_init_params": (C.c_int, [vp, C.c_ulonglong]),
            "sysu_gnn_set_params": (C.c_int, [vp, fp, C.c_int]),
            "sysu_gnn_get_params": (C.c_int, [vp, fp, C.c_int]),
            "sysu_gnn_apply": (C.c_int, [vp, dp, dp]),
            "sysu_gnn_add_pair": (C.c_int, [vp, dp, dp]),
            "sysu_gnn_loss_grad": (C.c_int, [vp, C.c_int, C.c_int, dp, fp, C.c_int]),
            "sysu_gnn_train": (C.c_int, [vp, C.c_int, C.c_double, C.c_int, dp]),
            "sysu_gnn_fcg": (C.c_int, [vp, dp, dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                       ip, dp, ip, ip, ip, dp]),
            "sysu_gnn_hidden": (C.c_int, [vp, dp, C.c_int, fp]),
            "sysu_gnn_time_apply": (C.c_int, [vp, dp, C.c_int, C.c_int, dp]),
            "sysu_gnn_last_error": (cp, []),
            "sysu_gnn_set_multigrid": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_double, ip, ip,
                                                 C.c_int]),
            "sysu_gnn_mg_apply": (C.c_int, [vp, dp, dp, C.c_int]),
            "sysu_mg_hierarchy": (C.c_int, [C.c_int, ip, ip, dp, C.c_double, C.c_int, C.c_int, ip, ip, lp]),
            "sysu_mg_level": (C.c_int, [C.c_int, ip, ip, dp, C.c_double, C.c_int, C.c_int, ip, ip, ip, dp]),
            "sysu_mg_last_error": (cp, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def pinned_empty(n: int) -> np.ndarray:
    """A float64 array of n values in page-locked host memory (freed with the array)."""
    import weakref

    L = lib()
    ptr = L.sysu_host_alloc(max(int(n), 1) * 8)
    if not ptr:
        raise SysuError(2, "page-locked host allocation failed")
    buf = (C.c_double * max(int(n), 1)).from_address(ptr)
    arr = np.ctypeslib.as_array(buf)[:n]
    weakref.finalize(arr, L.sysu_host_free, ptr)
    return arr


def check(code: int) -> None:
    if code != 0:
        raise SysuError(code, lib().sysu_last_error().decode())


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Case:
    """Host-only view of a case (parsed param.in + mesh + geometry); needs no GPU."""

    def __init__(self, param_path: str):
        self._h = C.c_void_p()
        check(lib().sysu_case_load(param_path.encode(), C.byref(self._h)))

    def close(self):
        if self._h:
            lib().sysu_case_free(self._h)
            self._h = C.c_void_p()

    __del__ = close

    def info(self) -> dict:
        out = (C.c_long * 12)()
        check(lib().sysu_case_info(self._h, out, 12))
        keys = ["Ncel", "Nfac", "Nbnd", "Nvrt", "NCoupledBnd", "solid_Ncel", "solid_Nfac", "solid_Nbnd",
                "solid_Nvrt", "solid_NCoupledBnd", "has_solid", "coupled_rid"]
        return dict(zip(keys, list(out)))

    def array(self, name: str) -> np.ndarray:
        L = lib()
        nbytes = L.sysu_case_array(self._h, name.encode(), None, 0)
        if nbytes < 0:
            raise KeyError(name)
        is_int = any(name.endswith(s) for s in ("nface", "face", "nbr", "rid", "vert", "c1", "c2", "bnd"))
        if name.endswith("vert") and name in ("vert", "solid_vert"):
            is_int = False
        dt = np.int32 if is_int else np.float64
        out = np.empty(nbytes // np.dtype(dt).itemsize, dtype=dt)
        L.sysu_case_array(self._h, name.encode(), out.ctypes.data_as(C.c_void_p), nbytes)
        return out

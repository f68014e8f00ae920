"""Learned preconditioner for symmetric systems (the p' equation): a 4-layer,
width-32 message-passing network over the matrix graph, trained on the GPU,
used inside flexible CG with a Jacobi fallback.  Thin ctypes mirror of the
sysu_gnn_* entry points of include/sysu_cfd.h; no counterpart in the
reference (its p' solve is CG + SSOR, navier_pressure.cpp:29)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

# flat parameter layout (FP32): [e(32) c(32)] [W_l (64 x 32, input-major), b_l (32)] x 4 [w_d(32) b_d]
WIDTH, LAYERS = 32, 4
OFF_ENC = 0
OFF_LAYER = 64
LAYER_STRIDE = 64 * 32 + 32
OFF_DEC = OFF_LAYER + LAYERS * LAYER_STRIDE
NPARAM = OFF_DEC + 33


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class LearnedPreconditioner:
    """Network + flexible CG on one CSR matrix held on the GPU."""

    def __init__(self, rowptr, col, val, capacity: int = 32):
        L = _lib.lib()
        if L.sysu_gnn_num_params() != NPARAM:
            raise RuntimeError("parameter layout mismatch with the library")
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        self.n = len(self.rowptr) - 1
        h = C.c_void_p()
        self._check(L.sysu_gnn_create(self.n, _ip(self.rowptr), _ip(self.col), _dp(self.val), capacity, C.byref(h)))
        self.h = h

    @staticmethod
    def _check(code):
        if code != 0:
            raise _lib.SysuError(code, _lib.lib().sysu_gnn_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            _lib.lib().sysu_gnn_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_values(self, val):
        """New values for the same pattern (rowptr, col of the constructor)."""
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        self._check(_lib.lib().sysu_gnn_set_values(self.h, _ip(self.rowptr), _ip(self.col), _dp(self.val)))

    def init_params(self, seed: int = 0):
        self._check(_lib.lib().sysu_gnn_init_params(self.h, seed))

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(NPARAM, np.float32)
        self._check(_lib.lib().sysu_gnn_get_params(self.h, _fp(p), NPARAM))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(_lib.lib().sysu_gnn_set_params(self.h, _fp(p), len(p)))

    def apply(self, r) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros(self.n)
        self._check(_lib.lib().sysu_gnn_apply(self.h, _dp(r), _dp(z)))
        return z

    def set_multigrid(self, on: bool = True, theta: float = 0.25, omega: float = 0.8, gamma: float = 1.8):
        """Attach (or detach) the aggregation-multigrid cycle: fcg() is then
        preconditioned by the V-cycle whose finest post-smoother is the network
        (use_gnn) or Jacobi, and add_pair() stores post-smoother pairs.  Returns
        the rows of each level."""
        lev = C.c_int()
        rows = (C.c_int * 16)()
        self._check(_lib.lib().sysu_gnn_set_multigrid(self.h, 1 if on else 0, theta, omega, gamma, C.byref(lev),
                                                      rows, 16))
        return [rows[i] for i in range(lev.value)] if on else []

    def mg_apply(self, r, use_gnn: bool = False) -> np.ndarray:
        """One application of the attached cycle, z = M(r)."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros(self.n)
        self._check(_lib.lib().sysu_gnn_mg_apply(self.h, _dp(r), _dp(z), 1 if use_gnn else 0))
        return z

    def hidden(self, r, layer: int) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        h = np.zeros((self.n, WIDTH), np.float32)
        self._check(_lib.lib().sysu_gnn_hidden(self.h, _dp(r), layer, _fp(h)))
        return h

    def add_pair(self, r, e):
        r = np.ascontiguousarray(r, dtype=np.float64)
        e = np.ascontiguousarray(e, dtype=np.float64)
        self._check(_lib.lib().sysu_gnn_add_pair(self.h, _dp(r), _dp(e)))

    def loss_grad(self, k: int = 0, loss_kind: int = 0):
        loss = C.c_double()
        g = np.zeros(NPARAM, np.float32)
        self._check(_lib.lib().sysu_gnn_loss_grad(self.h, k, loss_kind, C.byref(loss), _fp(g), NPARAM))
        return loss.value, g

    def train(self, steps: int, lr: float = 1e-3, loss_kind: int = 0) -> np.ndarray:
        losses = np.zeros(max(steps, 1))
        self._check(_lib.lib().sysu_gnn_train(self.h, steps, lr, loss_kind, _dp(losses)))
        return losses[:steps]

    def fcg(self, b, x0=None, maxit: int = 10000, eps: float = 1e-8, inner_tol: float = 0.1,
            use_gnn: bool = True, stall_max: int = 30):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        it, st, fb, ref = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        res, sec = C.c_double(), C.c_double()
        self._check(_lib.lib().sysu_gnn_fcg(self.h, _dp(b), _dp(x), 1 if x0 is None else 0, maxit, eps, inner_tol,
                                            1 if use_gnn else 0, stall_max, C.byref(it), C.byref(res),
                                            C.byref(st), C.byref(fb), C.byref(ref), C.byref(sec)))
        return x, {"iters": it.value, "res": res.value, "status": st.value, "fallback_at": fb.value,
                   "refinements": ref.value, "seconds": sec.value}

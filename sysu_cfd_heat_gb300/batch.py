"""Many independent SIMPLE cases advanced together in one CUDA graph, with the
SM-share autotuner (ctypes mirror of the sysu_batch_* entry points of
include/sysu_cfd.h).  No counterpart in the reference, which runs one case per
process."""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence

import numpy as np

from ._lib import SysuError, check, lib
from .solver import NavierStokesSolver

DEFAULT_CAPS = (1, 2, 4, 8, 16, 32, 64, 152)


class CaseBatch:
    def __init__(self, params: Sequence[str], options: Optional[Dict[str, float]] = None):
        L = lib()
        arr = (C.c_char_p * len(params))(*[p.encode() for p in params])
        h = C.c_void_p()
        check(L.sysu_batch_create(len(params), arr, C.byref(h)))
        self._h = h
        self.cases: List[NavierStokesSolver] = [NavierStokesSolver._borrow(L.sysu_batch_case(h, k))
                                                for k in range(len(params))]
        for s in self.cases:
            for k, v in (options or {}).items():
                s.set_option(k, v)

    def close(self):
        if self._h:
            for s in self.cases:
                s.close()
            lib().sysu_batch_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.cases)

    def tune(self, candidates: Sequence[int] = DEFAULT_CAPS) -> dict:
        n = len(self.cases)
        cand = (C.c_int * len(candidates))(*candidates)
        caps = (C.c_int * n)()
        alone = np.zeros(n)
        full = np.zeros(n)
        mk = C.c_double()
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        check(lib().sysu_batch_tune(self._h, cand, len(candidates), caps, dp(alone), dp(full), C.byref(mk)))
        return {"sm_cap": list(caps), "ms_alone": alone.tolist(), "ms_full": full.tolist(),
                "measured_makespan_ms": mk.value}

    def set_caps(self, caps: Sequence[int]):
        arr = (C.c_int * len(caps))(*caps)
        check(lib().sysu_batch_set_caps(self._h, arr))

    def capture(self):
        check(lib().sysu_batch_capture(self._h))

    def replay(self, n: int) -> float:
        ms = C.c_double()
        check(lib().sysu_batch_replay(self._h, n, C.byref(ms)))
        return ms.value

    def check(self):
        check(lib().sysu_batch_check(self._h))

    def run_sequential(self, n: int) -> float:
        ms = C.c_double()
        check(lib().sysu_batch_run_sequential(self._h, n, C.byref(ms)))
        return ms.value

"""Device-side solve loops (CUDA graph WHILE nodes, graph_loop.cu): the loop's
last kernel ends it when the solve's stop flag is set or after the bound, so a loop
whose flag is never set still ends (sysu_graph_loop_selftest runs such a graph)."""
import ctypes as C

import pytest

from sysu_cfd_heat_gb300._lib import lib

pytestmark = pytest.mark.gpu


def _bodies(bound, stop_at):
    n = C.c_int(-1)
    rc = lib().sysu_graph_loop_selftest(bound, stop_at, C.byref(n))
    assert rc == 0, lib().sysu_csr_last_error()
    return n.value


@pytest.mark.parametrize("bound,stop_at", [(1, 0), (7, 0), (64, 0), (10, 3), (10, 1), (4, 9), (5, 5)])
def test_loop_ends_at_flag_or_bound(bound, stop_at):
    expect = bound if stop_at <= 0 else min(stop_at, bound)
    assert _bodies(bound, stop_at) == expect


def test_loop_rejects_a_bound_below_one():
    n = C.c_int(0)
    assert lib().sysu_graph_loop_selftest(0, 0, C.byref(n)) != 0

"""Input validation runs on the host: ecpgb_layout parses a system without a
GPU and refuses the documented out-of-range inputs with a message."""
import ctypes as ct

import numpy as np
import pytest

from libecp_gb300 import workloads as W


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


def layout(eg, s):
    cs = eg.c_system(s)
    nu, nv = ct.c_longlong(0), ct.c_longlong(0)
    rc = eg.lib().ecpgb_layout(ct.byref(cs), ct.byref(nu), ct.byref(nv))
    return rc, nu.value, nv.value, (eg.last_error() if rc else "")


def test_valid_system_has_a_layout(eg):
    s = W.random_system(3, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    rc, nu, nv, _ = layout(eg, s)
    assert rc == 0 and nu == s.n_pairs * 2 and nv > 0


@pytest.mark.parametrize("order,ok", [(383, False), (384, True), (2048, True), (8190, True), (8191, False)])
def test_large_grid_order_range(eg, order, ok):
    """largeGridOrder 384..8190: the grid has 2^floor(log2(order + 1)) - 1
    points, at most 4095 (8191 would give 8191)."""
    s = W.random_system(3, n_atoms=2, n_centres=1, lmax_basis=1, lmax_ecp=2)
    s.largeGridOrder = order
    rc, _, _, msg = layout(eg, s)
    assert (rc == 0) == ok, msg
    if not ok:
        assert "largeGridOrder" in msg and "384..8190" in msg


def test_basis_l_and_contraction_limits(eg):
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=[(0, [(2.0, 1.0, 1.0)])], shells=[(5, [(1.0, 1.0)])])
    rc, _, _, msg = layout(eg, b.build("h shell"))
    assert rc and "basis l=5" in msg
    b = W._Builder()
    prims = [(0.1 * (i + 1), 1.0) for i in range(17)]
    b.atom([0.0, 0.0, 0.0], ecp=[(0, [(2.0, 1.0, 1.0)])], shells=[(0, prims)])
    rc, _, _, msg = layout(eg, b.build("K=17"))
    assert rc and "contraction 17" in msg


def test_derivative_order_limit(eg):
    s = W.random_system(3, n_atoms=2, n_centres=1, lmax_basis=1, lmax_ecp=2)
    s.derivative = 3
    rc, _, _, msg = layout(eg, s)
    assert rc and "derivative order 3" in msg

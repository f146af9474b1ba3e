"""Caller's Cartesian order (libECP_init's lmax and shellOrdering,
src/libecp.c:159-165): blocks against a fixture recorded from the reference
with libint's order reversed in every shell, through the callback interface
and the batched blocks of both FP64 paths; the matrix in that order; the
reference's refusal of an order that does not reach far enough."""
import numpy as np
import pytest

import libecp_gb300
from libecp_gb300 import workloads as W
from tests.helpers import TOL_ABS, load_golden, ordered_golden_files
from tests.test_gpu_parity import assert_blocks_match

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    libecp_gb300.lib()
    return libecp_gb300


@pytest.mark.parametrize("name", ordered_golden_files())
def test_callback_interface(eg, name):
    s, z = load_golden(name)
    rc, meta, data = eg.calculate_blocks_via_callback(s)
    assert rc == 0
    assert_blocks_match(meta, data, z["meta"], z["data"])


@pytest.mark.parametrize("mode_name", ["ECPGB_FP64", "ECPGB_FAST"])
@pytest.mark.parametrize("name", ordered_golden_files())
def test_blocks(eg, name, mode_name):
    s, z = load_golden(name)
    meta, data = eg.blocks(s, mode=getattr(eg, mode_name))
    assert_blocks_match(meta, data, z["meta"], z["data"])


def test_matrix_is_the_permuted_matrix(eg):
    s, z = load_golden(ordered_golden_files()[0])
    rc, Io, _ = eg.get_integrals_info(s)
    s2, _ = load_golden(ordered_golden_files()[0])
    s2.ordering = None
    rc, Id, _ = eg.get_integrals_info(s2)
    # AO index map: within each shell the order is reversed
    perm, ao = [], 0
    for l in s.lBS:
        n = (l + 1) * (l + 2) // 2
        perm += list(range(ao + n - 1, ao - 1, -1))
        ao += n
    full = lambda U: U + U.T - np.diag(np.diag(U))
    assert np.abs(full(Io) - full(Id)[np.ix_(perm, perm)]).max() <= TOL_ABS


def test_order_too_short_is_refused(eg):
    s = W.random_system(2, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    need = s.max_l_ecp() + 2 * s.max_l_basis()
    s.ordering = eg.libint_ordering(need - 1)
    s.ordering_lmax = need - 1
    with pytest.raises(RuntimeError, match="shellOrdering"):
        eg.blocks(s)
    with pytest.raises(RuntimeError, match="libECP_init"):
        eg.calculate_blocks_via_callback(s)

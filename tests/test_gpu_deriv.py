"""Nuclear-derivative blocks (libECP_init with n = 1, 2): every shifted
(shell pair, centre) block of the reference's derivative scheme
(src/libecp.c:240-374) against fixtures recorded from the unmodified
reference, through the drop-in callback interface and through the batched
blocks interface of both FP64 paths, at the FP64 bar."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W
from tests.helpers import TOL_ABS, deriv_golden_files, load_golden
from tests.test_gpu_parity import assert_blocks_match

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


@pytest.mark.parametrize("name", deriv_golden_files())
def test_callback_interface_matches_reference(eg, name):
    s, z = load_golden(name)
    assert s.derivative in (1, 2)
    rc, meta, data = eg.calculate_blocks_via_callback(s)
    assert rc == 0
    assert_blocks_match(meta, data, z["meta"], z["data"])


@pytest.mark.parametrize("mode_name", ["ECPGB_FP64", "ECPGB_FAST"])
@pytest.mark.parametrize("name", deriv_golden_files())
def test_blocks_match_reference(eg, name, mode_name):
    s, z = load_golden(name)
    meta, data = eg.blocks_deriv(s, mode=getattr(eg, mode_name))
    assert_blocks_match(meta, data, z["meta"], z["data"])


def test_order_zero_is_the_plain_blocks(eg):
    s = W.random_system(3, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=4)
    m0, d0 = eg.blocks(s)
    m1, d1 = eg.blocks_deriv(s)
    assert np.array_equal(m0, m1[:, [0, 1, 2, 4, 5, 6, 8, 9]]) and np.array_equal(d0, d1)
    assert not m1[:, [3, 7]].any()


def test_derivative_jobs_batched_and_resident(eg):
    s = W.batched_cluster(0).subset(centres=[0, 1], basis_atoms=range(5))
    s.derivative = 1
    v64, o64, st64, _ = eg.raw_blocks(s, eg.ECPGB_FP64)
    vf, of, stf, _ = eg.raw_blocks(s, eg.ECPGB_FAST)
    assert np.array_equal(st64, stf) and np.array_equal(o64, of)
    assert np.abs(v64 - vf).max() <= TOL_ABS
    j = eg.Job(s, mode=eg.ECPGB_FAST)
    assert j.launches_per_run() == (9 if j.config()["queue"] and j.config()["screen"] else 6)
    j.run(1)
    v, st = j.blocks()
    assert np.array_equal(st, stf) and np.abs(v - vf).max() <= TOL_ABS
    j.close()


def test_matrix_refuses_derivatives(eg):
    s = W.example_like(0)
    s.derivative = 1
    with pytest.raises(RuntimeError, match="derivative order 0"):
        eg.get_integrals_info(s, mode=eg.ECPGB_FAST)

"""Spherical output: the GPU's T(la) B T(lb)^T of every block equals the same
product formed on the host from the Cartesian blocks, for plain, derivative
and caller-ordered jobs."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W
from libecp_gb300.workloads import ncart

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


def host_sph(eg, meta, data, n):
    out, off = [], 0
    for m in meta:
        if n:
            la, ha, lb, hb = m[2], m[3], m[6], m[7]
            la, lb = eg.block_l(n, la, lb, ha, hb)
        else:
            la, lb = m[2], m[5]
        B = data[off:off + ncart(la) * ncart(lb)].reshape(ncart(la), ncart(lb))
        off += ncart(la) * ncart(lb)
        out.append((eg.cart2sph(la) @ B @ eg.cart2sph(lb).T).ravel())
    return np.concatenate(out)


@pytest.mark.parametrize("deriv", [0, 1])
@pytest.mark.parametrize("mode_name", ["ECPGB_FP64", "ECPGB_FAST"])
def test_sph_blocks(eg, deriv, mode_name):
    s = W.random_system(3, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=4)
    s.derivative = deriv
    mode = getattr(eg, mode_name)
    mc, dc = (eg.blocks_deriv(s, mode=mode) if deriv else eg.blocks(s, mode=mode))
    ms, ds = eg.blocks_sph(s, mode=mode)
    assert np.array_equal(mc, ms)
    ref = host_sph(eg, mc, dc, deriv)
    assert np.abs(ds - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())

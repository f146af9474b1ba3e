"""Rotation invariance (a known-answer property of the integrals, independent
of the reference): rotating every atom by R turns each Cartesian block V into
T(la) V T(lb)^T, where T(l)[a][a'] are the coefficients of the monomial a of
R x in the monomials a' of x; the semi-local projectors and the radial parts
are invariant.  Checked on both FP64 paths, s..d shells."""
import itertools

import numpy as np
import pytest

from libecp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


def cart(l):
    return [(l - i, i - j, j) for i in range(l + 1) for j in range(i + 1)]


def monomial_map(R, l):
    """T[a][a']: monomial a of (R x) expanded in monomials a' of x."""
    idx = {e: k for k, e in enumerate(cart(l))}
    T = np.zeros((len(idx), len(idx)))
    for a, (ax, ay, az) in enumerate(cart(l)):
        # (R x)_k^p = (sum_j R_kj x_j)^p: multiply out the 3 (ax + ay + az) linear factors
        factors = [R[0]] * ax + [R[1]] * ay + [R[2]] * az
        poly = {(0, 0, 0): 1.0}
        for f in factors:
            nxt = {}
            for e, c in poly.items():
                for j in range(3):
                    if f[j] == 0.0:
                        continue
                    e2 = list(e)
                    e2[j] += 1
                    nxt[tuple(e2)] = nxt.get(tuple(e2), 0.0) + c * f[j]
            poly = nxt
        for e, c in poly.items():
            T[a, idx[e]] += c
    return T


def rotation(seed):
    q = np.random.default_rng(seed).normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


@pytest.mark.parametrize("mode_name", ["ECPGB_FP64", "ECPGB_FAST"])
def test_rotated_blocks(eg, mode_name):
    mode = getattr(eg, mode_name)
    s = W.random_system(31, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    R = rotation(4)
    t = W.EcpSystem(**{f: getattr(s, f) for f in s.__dataclass_fields__})
    t.geometry = (s.geometry.reshape(-1, 3) @ R.T).ravel()
    m0, d0 = eg.blocks(s, mode=mode)
    m1, d1 = eg.blocks(t, mode=mode)
    assert np.array_equal(m0, m1)
    Ts = {l: monomial_map(R, l) for l in range(3)}
    off, worst, scale = 0, 0.0, np.abs(d0).max()
    for m in m0:
        la, lb = m[2], m[5]
        n = len(cart(la)) * len(cart(lb))
        V = d0[off:off + n].reshape(len(cart(la)), len(cart(lb)))
        Vr = d1[off:off + n].reshape(V.shape)
        worst = max(worst, np.abs(Ts[la] @ V @ Ts[lb].T - Vr).max())
        off += n
    assert worst <= 1e-9 * scale, (worst, scale)

"""The oracle (CPU restatement) pinned against the reference and against
mathematics.  CPU only."""
import ctypes as ct
import math

import numpy as np
import pytest

from libecp_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import golden_files, load_golden, one_centre_answers, one_centre_system

_D = ct.POINTER(ct.c_double)


@pytest.mark.parametrize("name", golden_files())
def test_oracle_reproduces_reference_fixtures(name):
    """Fixtures were produced by the unmodified reference; the oracle must give
    the same blocks in the same callback order (bit-for-bit where the libm and
    compiler match; 1e-12 relative elsewhere)."""
    s, z = load_golden(name)
    rc, meta, data = O.oracle_blocks(s)
    assert rc == 0
    assert np.array_equal(meta, z["meta"])
    ref = z["data"]
    assert np.all(np.abs(data - ref) <= 1e-12 + 1e-12 * np.abs(ref))
    if "matrix" in z:
        rc, I = O.oracle_matrix(s)
        assert np.all(np.abs(I - z["matrix"]) <= 1e-12 + 1e-12 * np.abs(z["matrix"]))


def test_oracle_matches_reference_live():
    """Where the reference was built in this container, compare live too."""
    if not O.ref_available():
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    for seed in (7, 8):
        s = W.random_system(seed, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3, kmax=2)
        rc1, m1, d1 = O.ref_blocks(s)
        rc2, m2, d2 = O.oracle_blocks(s)
        assert rc1 == rc2 == 0 and np.array_equal(m1, m2)
        assert np.max(np.abs(d1 - d2)) <= 1e-12 * max(1.0, np.max(np.abs(d1)))


def test_one_centre_known_answers():
    s, _, _ = one_centre_system()
    rc, I = O.oracle_matrix(s)
    assert rc == 0
    for (i, j), v in one_centre_answers().items():
        assert abs(I[i, j] - v) <= 1e-12 * max(1.0, abs(v)), (i, j, I[i, j], v)


def test_padding_adds_exactly_zero():
    """The zero-coefficient pad centre used to keep the reference in bounds
    changes no block of the original centres."""
    s = W.random_system(3, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    rc1, m1, d1 = O.oracle_blocks(s)
    rc2, m2, d2 = O.oracle_blocks(s.padded())
    assert rc1 == rc2 == 0
    assert np.array_equal(m1, m2) and np.array_equal(d1, d2)


def test_bessel_against_scipy():
    """K_l(z) = exp(-z) i_l(z) in all three branches of the evaluation."""
    sp = pytest.importorskip("scipy.special")
    L = O.oracle_lib()
    K = np.zeros(16)
    for z in (0.0, 5e-8, 0.003, 0.3, 1.7, 9.99, 15.9999, 16.0, 25.0, 80.0):
        assert L.oracle_bessel(10, z, 16, 1e-14, K.ctypes.data_as(_D)) == 0
        for l in range(11):
            ref = math.exp(-z) * sp.spherical_in(l, z) if z > 0 else (1.0 if l == 0 else 0.0)
            # the table's series stops on an absolute 1e-14 term, so small
            # values carry absolute, not relative, error
            tol = 1e-12 * abs(ref) + 2e-14
            if z < 1e-6 and l > 0:
                tol = max(tol, abs(ref) * z * 2)  # small-argument branch drops O(z^2) terms
            assert abs(K[l] - ref) <= tol, (z, l, K[l], ref)


def test_real_spherical_harmonics_orthonormal():
    L = O.oracle_lib()
    lmax = 5
    xg, wg = np.polynomial.legendre.leggauss(24)
    nphi = 48
    phis = (np.arange(nphi) + 0.5) * 2 * np.pi / nphi
    n = (lmax + 1) ** 2
    G = np.zeros((n, n))
    out = np.zeros(n)
    for x, w in zip(xg, wg):
        th = math.acos(x)
        for ph in phis:
            L.oracle_rsh(lmax, th, ph, out.ctypes.data_as(_D))
            G += w * (2 * np.pi / nphi) * np.outer(out, out)
    assert np.max(np.abs(G - np.eye(n))) < 1e-12


@pytest.mark.parametrize("which,npts,order", [(0, 128, 383), (1, 1024, 1023)])
def test_grids_integrate(which, npts, order):
    """Nested Gauss-Chebyshev grids: increasing abscissae and the full-grid
    rule int f = 16/(3(n+1)) sum w f (PS93 on (0, inf) after the Krack-Koster
    map, PSM92 on (-1, 1))."""
    L = O.oracle_lib()
    x, w = np.zeros(4096), np.zeros(4096)
    m = L.oracle_grid(which, npts, x.ctypes.data_as(_D), w.ctypes.data_as(_D))
    assert m == order
    x, w = x[:m], w[:m]
    assert np.all(np.diff(x) > 0)
    if which == 0:
        val, ref = 16 * np.sum(w * np.exp(-x ** 2)) / (3 * (m + 1)), math.sqrt(math.pi) / 2
    else:
        val, ref = 16 * np.sum(w / (1 + x ** 2)) / (3 * (m + 1)), math.pi / 2
    assert abs(val - ref) < 1e-12


def test_alternatives_leave_the_reference_branch_unchanged():
    """With decision tracking on, the primary blocks are exactly the
    oracle's; alternatives exist only for blocks whose quadratures took a
    decision within the noise bound, and the bound grows with kappa."""
    s = W.random_system(16, n_atoms=4, n_centres=2, lmax_basis=3, lmax_ecp=4, kmax=4,
                        elo=0.01, ehi=500.0)
    rc, m0, d0 = O.oracle_blocks(s)
    counts = []
    for kappa in (0.0, 16.0, 1e6):
        rc2, m, d, am, ad, sc = O.oracle_blocks_alt(s, kappa)
        assert np.all(sc >= np.array([np.max(np.abs(d[o:o + n])) for o, n in _spans(m)]) * (1 - 1e-12))
        assert rc2 == rc and np.array_equal(m, m0) and np.array_equal(d, d0)
        counts.append(len(am))
        keys = {tuple(r) for r in m.tolist()}
        assert all(tuple(r) in keys for r in am.tolist())
    assert counts[0] == 0 and counts[0] <= counts[1] <= counts[2] and counts[2] > 0
    # the matcher: a block equal to an alternative passes, a perturbed one does not
    rc2, m, d, am, ad, sc = O.oracle_blocks_alt(s, 1e6)
    n0 = ((am[0][2] + 1) * (am[0][2] + 2) // 2) * ((am[0][5] + 1) * (am[0][5] + 2) // 2)
    off = 0
    for row in m:
        n = ((row[2] + 1) * (row[2] + 2) // 2) * ((row[5] + 1) * (row[5] + 2) // 2)
        if np.array_equal(row, am[0]):
            break
        off += n
    g = d.copy()
    g[off:off + n0] = ad[:n0]
    bar = lambda r: 1e-10 + 1e-13 * float(np.max(np.abs(r)))
    res = O.match_blocks(m, g, m, d, am, ad, bar)
    assert not res["failures"]
    g[off] += 1.0
    res = O.match_blocks(m, g, m, d, am, ad, bar)
    assert len(res["failures"]) == 1


def _spans(meta):
    off = 0
    for m in meta:
        n = ((m[2] + 1) * (m[2] + 2) // 2) * ((m[5] + 1) * (m[5] + 2) // 2)
        yield off, n
        off += n


@pytest.mark.parametrize("name", ["cluster_subset_s0", "random_g_s101", "random_fL5_s200"])
def test_division_free_ps93_test_takes_the_reference_decision(name):
    """The GPU kernels test the PS93 error estimate as 16 d < tol 3 n instead of
    16 d / (3 n) < tol.  The two forms can differ only where 16 d / (3 n) lies
    within half an ulp of tol; on every small-grid decision of these fixtures'
    systems (every level the reference tests) they take the same branch."""
    s, _ = load_golden(name + ".npz")
    rc, meta, data, st = O.oracle_blocks(s, with_stats=True)
    assert rc == 0
    assert st["ps93_decisions"] > 1000
    assert st["ps93_divfree_flips"] == 0, st

"""Shared helpers for the tests (no GPU needed to import)."""
import os
from math import gamma, pi

import numpy as np

from libecp_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
# Parity bar of the FP64 path against the FP64 reference / oracle.
TOL_ABS = 1e-10


def golden_files():
    """Fixtures of derivative order 0 in libint's Cartesian order."""
    return sorted(f for f in os.listdir(GOLDEN_DIR)
                  if f.endswith(".npz") and not f.startswith(("deriv", "ordered")))


def ordered_golden_files():
    """Fixtures in a caller's Cartesian order (libECP_init's shellOrdering)."""
    return sorted(f for f in os.listdir(GOLDEN_DIR) if f.endswith(".npz") and f.startswith("ordered"))


def deriv_golden_files():
    """Fixtures of the nuclear-derivative blocks (order 1 and 2)."""
    return sorted(f for f in os.listdir(GOLDEN_DIR) if f.endswith(".npz") and f.startswith("deriv"))


def load_golden(name):
    import sys
    sys.path.insert(0, GOLDEN_DIR)
    from make_golden import load
    return load(os.path.join(GOLDEN_DIR, name))


def one_centre_system():
    """ECP and basis on one atom: closed-form answers exist (see one_centre_answers)."""
    b = W._Builder()
    ecp = [(0, [(2.0, 3.0, 1.3)]), (1, [(2.0, -2.0, 0.7)]), (2, [(2.0, 1.5, 2.1), (1.0, 0.5, 0.4)])]
    za, ca, zb, cb = 0.8, 0.6, 1.7, 0.9
    b.atom([0.0, 0.0, 0.0], ecp=ecp, shells=[(0, [(ca, za)]), (1, [(cb, zb)]), (0, [(cb, zb)])])
    return b.build("one_centre"), ecp, (za, ca, zb, cb)


def one_centre_answers():
    """<a|U|b> with a, b and U on one centre:
    4 pi/(2l+1) c_a c_b sum_terms d Gamma((n+2l+1)/2) / (2 p^((n+2l+1)/2)),
    p = zeta_a + zeta_b + a, over the local terms and the semi-local channel l
    of the shells (the radial Jacobian r^2 is part of the ECP's r^n)."""
    _, ecp, (za, ca, zb, cb) = one_centre_system()

    def rad(terms, p0, k):
        return sum(d * gamma((n + k + 1) / 2) / (2 * (p0 + a) ** ((n + k + 1) / 2))
                   for n, d, a in terms)
    loc, ch0, ch1 = ecp[2][1], ecp[0][1], ecp[1][1]
    return {
        (0, 0): 4 * pi * ca * ca * (rad(loc, 2 * za, 0) + rad(ch0, 2 * za, 0)),
        (0, 4): 4 * pi * ca * cb * (rad(loc, za + zb, 0) + rad(ch0, za + zb, 0)),
        (1, 1): 4 * pi / 3 * cb * cb * (rad(loc, 2 * zb, 2) + rad(ch1, 2 * zb, 2)),
        (1, 2): 0.0, (0, 1): 0.0,
    }


def max_rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


# Bar for configurations with g shells and large exponents (elements up to
# 6e9; the shift onto A and B sums terms up to ~1e7 times larger than the
# block).  Any correct FP64 evaluation of a block differs from another by a
# few units of 2^-53 times the block's scale -- its largest element
# evaluated over absolute values, which the oracle returns with
# oracle_blocks_alt (measured: at most 3.7 units between the oracle and
# either GPU path on the mixed batch and the sweep).  The bar is TOL_ABS
# plus 128 units; blocks without cancellation and below 1e3 keep the 1e-10
# absolute bar.
SCALE_UNITS = 128.0


def bar_scaled(ref_block, scale) -> float:
    return TOL_ABS + SCALE_UNITS * 2.0 ** -53 * float(scale)


# Bar of the mixed-precision path: double-single carries about 2^-48 of a
# block's scale where FP64 carries 2^-53, so 2^-44 of the scale replaces the
# FP64 bar's 128 units of 2^-53 (on the 50-centre cluster, where the scales
# stay below 1e6, the two differ by less than 1e-10).
def bar_mixed(ref_block, scale) -> float:
    return TOL_ABS + 2.0 ** -44 * float(scale)


# Rounding-noise bound (in units of 2^-53 times the sum of |w f| of a
# quadrature) within which the oracle marks a convergence decision as
# ambiguous and offers the inverted branch (oracle_blocks_alt).  The GPU
# paths evaluate the integrands with other (correct) roundings: CUDA's exp,
# the batched path's Horner Bessel rows and table exp, contracted multiply-adds.
KAPPA_FP64 = 128.0


def size_preserving_subset(s, centres, basis_atoms):
    """s.subset with, in addition, one atom carrying a shell of the system's
    largest l and the centre with its largest ECP L, so that the reference's
    global table sizes -- and with them the values its fallbacks read from
    stale buffers -- are those of the full system."""
    lmax, Lmax = s.max_l_basis(), s.max_l_ecp()
    starts = np.concatenate([[0], np.cumsum(s.shellsBS)]).astype(int)
    G = next(a for a in range(s.n_atoms) if np.any(s.lBS[starts[a]:starts[a + 1]] == lmax))
    est = np.concatenate([[0], np.cumsum(s.shellsECP)]).astype(int)
    CL = next(a for a in range(s.n_atoms)
              if s.shellsECP[a] and int(np.max(s.lECP[est[a]:est[a + 1]])) == Lmax)
    return s.subset(centres=sorted(set(centres) | {CL}), basis_atoms=sorted(set(basis_atoms) | {G}))

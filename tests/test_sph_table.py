"""The Cartesian -> real spherical matrices (no GPU): with Cartesian functions
each normalised on its own, T(l) S(l) T(l)^T = 1 (Schlegel and Frisch,
Int. J. Quantum Chem. 54 (1995) 83), S(l) the overlap of the normalised
Cartesian functions of one shell (same centre and exponent)."""
import math

import numpy as np
import pytest


def dfact(n):
    return 1 if n <= 0 else n * dfact(n - 2)


def cart(l):
    return [(l - i, i - j, j) for i in range(l + 1) for j in range(i + 1)]


def overlap(l):
    fs = cart(l)
    S = np.zeros((len(fs), len(fs)))
    norm = [math.sqrt(dfact(2 * a - 1) * dfact(2 * b - 1) * dfact(2 * c - 1)) for a, b, c in fs]
    for i, (a, b, c) in enumerate(fs):
        for j, (d, e, f) in enumerate(fs):
            if (a + d) % 2 or (b + e) % 2 or (c + f) % 2:
                continue
            S[i, j] = dfact(a + d - 1) * dfact(b + e - 1) * dfact(c + f - 1) / (norm[i] * norm[j])
    return S


@pytest.mark.parametrize("l", [0, 1, 2, 3, 4])
def test_cart2sph_orthonormal(l):
    import libecp_gb300 as eg
    T = eg.cart2sph(l)
    assert T.shape == (2 * l + 1, (l + 1) * (l + 2) // 2)
    assert np.abs(T @ overlap(l) @ T.T - np.eye(2 * l + 1)).max() < 1e-13

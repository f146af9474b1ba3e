"""Device-side consumers: the energy E = sum D V of a density matrix and its
nuclear gradient assembled on the GPU from the derivative-order-1 blocks.
The gradient is checked against central finite differences of the energy
(getIntegrals at displaced geometries), translational invariance (the atom
gradients sum to zero) and across the two FP64 paths."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


def density(dim, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(dim, dim)) / dim
    return X + X.T


def energy_of_matrix(I, D):
    U = np.triu(I)
    return float((D * (U + U.T - np.diag(np.diag(U)))).sum())


def uncontracted(seed, n_atoms, n_centres, lmax_basis, lmax_ecp):
    """A random system with one primitive per shell.  With contracted shells the
    reference's large-grid fallback integrates, beyond a primitive pair's break
    point, the tables an earlier pair of the same unit left behind
    (src/type2.c:549-601); where that break point moves with the geometry the
    blocks jump, so finite differences of E measure those jumps, not the
    derivative.  With one primitive per shell there is no earlier pair."""
    rng = np.random.default_rng(seed)
    b = W._Builder()
    for i in range(n_atoms):
        ecp = W._ecp_channels(rng, lmax_ecp if i == 0 else int(rng.integers(1, lmax_ecp + 1)), 2) \
            if i < n_centres else None
        shells = [(int(rng.integers(0, lmax_basis + 1)), [(float(rng.uniform(0.3, 1.0)),
                                                            float(np.exp(rng.uniform(np.log(0.1), np.log(5.0)))))])
                  for _ in range(int(rng.integers(1, 4)))]
        b.atom(rng.uniform(-1.6, 1.6, 3), ecp=ecp, shells=shells)
    return b.build(f"uncontracted({seed})")


SYSTEMS = [
    ("spd", lambda: uncontracted(21, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)),
    ("f-shells", lambda: uncontracted(22, n_atoms=2, n_centres=2, lmax_basis=3, lmax_ecp=4)),
    ("one-ecp", lambda: uncontracted(23, n_atoms=4, n_centres=1, lmax_basis=1, lmax_ecp=2)),
]


@pytest.mark.parametrize("name,make", SYSTEMS, ids=[n for n, _ in SYSTEMS])
def test_gradient_matches_finite_differences(eg, name, make):
    s = make()
    D = density(s.dim, 5)
    E, g = eg.gradient(s, D)
    rc, I, _ = eg.get_integrals_info(s)
    assert abs(E - energy_of_matrix(I, D)) <= 1e-10 * max(1.0, abs(E))
    assert np.abs(g.sum(axis=0)).max() <= 1e-9 * max(1.0, np.abs(g).max())  # translational invariance
    h = 1e-4
    fd = np.zeros_like(g)
    for a in range(s.n_atoms):
        for k in range(3):
            vals = []
            for sign in (1, -1):
                t = W.EcpSystem(**{f: getattr(s, f) for f in s.__dataclass_fields__})
                t.geometry = s.geometry.copy()
                t.geometry[3 * a + k] += sign * h
                vals.append(energy_of_matrix(eg.get_integrals_info(t)[1], D))
            fd[a, k] = (vals[0] - vals[1]) / (2 * h)
    scale = max(1.0, np.abs(g).max())
    assert np.abs(fd - g).max() <= 2e-5 * scale, (np.abs(fd - g).max(), scale)


def test_paths_agree_and_energy_only(eg):
    s = W.batched_cluster(0).subset(centres=[0, 1, 2], basis_atoms=range(6))
    D = density(s.dim, 9)
    E1, g1 = eg.gradient(s, D, mode=eg.ECPGB_FP64)
    E2, g2 = eg.gradient(s, D, mode=eg.ECPGB_FAST)
    assert abs(E1 - E2) <= 1e-10 * max(1.0, abs(E1))
    assert np.abs(g1 - g2).max() <= 1e-9 * max(1.0, np.abs(g1).max())

"""Seeded workload generators: determinism and shapes.  CPU only."""
import numpy as np

from libecp_gb300 import workloads as W


def test_example_like_shape():
    s = W.example_like(0)
    assert s.n_atoms == 5 and s.n_shells == 12 and s.n_pairs == 78 and s.n_centres == 1
    assert s.dim == 40 and not s.needs_pad()
    assert list(s.lECP) == [0, 1, 2, 3, 4] and list(s.KECP) == [3] * 5


def test_batched_cluster_shape():
    s = W.batched_cluster(0)
    assert s.n_centres == 50 and s.n_shells == 63 and s.n_pairs == 2016
    assert s.n_units == 100800
    assert s.max_l_basis() <= 3 and s.max_l_ecp() == 4 and not s.needs_pad()
    assert 1 <= s.KBS.min() and s.KBS.max() <= 8


def test_generators_are_deterministic():
    for make in (lambda: W.example_like(3), lambda: W.batched_cluster(2),
                 lambda: W.random_system(5), lambda: W.mixed_batch(1, n_shells=40),
                 lambda: W.large_sweep(1, n_shells=30)):
        a, b = make(), make()
        for k in ("geometry", "lECP", "aECP", "dECP", "lBS", "KBS", "aBS", "dBS"):
            assert np.array_equal(getattr(a, k), getattr(b, k))


def test_subset_keeps_geometry_and_order():
    s = W.batched_cluster(0)
    t = s.subset(centres=[3], basis_atoms=[0, 5])
    assert t.n_atoms == s.n_atoms and np.array_equal(t.geometry, s.geometry)
    assert t.n_centres == 1 and t.shellsECP[3] == s.shellsECP[3]
    assert t.n_shells == s.shellsBS[0] + s.shellsBS[5]


def test_padding_raises_global_maxima_only():
    s = W.random_system(101, n_atoms=3, n_centres=2, lmax_basis=4, lmax_ecp=3, kmax=2)
    assert s.needs_pad()
    p = s.padded()
    assert not p.needs_pad()
    assert p.n_atoms == s.n_atoms + 1 and p.shellsBS[-1] == 0 and p.dECP[-1] == 0.0

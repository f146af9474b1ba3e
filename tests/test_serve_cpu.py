"""Host logic of the serving driver (no GPU): the Poisson arrival process,
the request stream's shapes and the latency summary."""
import numpy as np

from libecp_gb300 import serve


def test_poisson_arrivals_rate_and_order():
    t = serve.poisson_arrivals(200.0, 30.0, seed=3)
    assert np.all(np.diff(t) > 0) and t[0] >= 0 and t[-1] < 30.0
    assert abs(len(t) / 30.0 - 200.0) < 200.0 * 0.05  # 6000 arrivals: 5 % is > 3 sigma
    gaps = np.diff(t)
    assert abs(gaps.mean() - 1 / 200.0) < 0.05 / 200.0
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.05  # exponential gaps: cv = 1
    assert np.array_equal(t, serve.poisson_arrivals(200.0, 30.0, seed=3))


def test_request_stream_shapes():
    systems = serve.request_stream(40, seed=1)
    again = serve.request_stream(40, seed=1)
    for s, s2 in zip(systems, again):
        assert s.n_atoms == s2.n_atoms and s.dim == s2.dim
        assert 5 <= s.n_atoms <= 200
        centres = int(np.count_nonzero(np.asarray(s.shellsECP) > 0))
        assert 1 <= centres <= min(40, s.n_atoms)
        assert max(s.lBS) <= 3 and 1 <= min(s.KBS) and max(s.KBS) <= 6
    sizes = [s.n_atoms for s in systems]
    assert min(sizes) < 30 < max(sizes)  # log-uniform over 5..200


def test_percentiles():
    p = serve.percentiles(np.arange(1, 101))
    assert p["p50"] == 50.5 and abs(p["p99"] - 99.01) < 1e-9 and p["max"] == 100
    assert serve.percentiles([])["p99"] is None

"""The request server: continuous batching on one GPU.

Every served result must equal, bit for bit, the same system run alone through
ecpgb_getIntegrals with the same mode (a job runs the same kernels and launch
configuration in the mix as alone); admission respects the device-memory
budget; jobs overlap (several in flight at once); a job larger than the
budget fails cleanly without stopping the others."""
import numpy as np
import pytest

from libecp_gb300 import serve
from libecp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


@pytest.fixture(scope="module")
def stream():
    rng = np.random.default_rng(11)
    systems = []
    for i in range(24):
        atoms = int(rng.integers(5, 40))
        systems.append(W.serving_molecule(rng, atoms, int(rng.integers(1, min(atoms, 12) + 1))))
    return systems


@pytest.mark.parametrize("mode_name", ["ECPGB_FAST", "ECPGB_FP64"])
def test_results_identical_alone_and_in_the_mix(eg, stream, mode_name):
    mode = getattr(eg, mode_name)
    alone = [eg.get_integrals_info(s, mode=mode)[1] for s in stream]
    with eg.Server(mode=mode, budget_bytes=4 << 30, slots=6) as sv:
        ids = [sv.submit(s) for s in stream]  # a burst: later jobs start while earlier run
        out = [sv.wait(i) for i in ids]
        st = sv.stats()
    assert st["completed"] == len(stream) and st["failed"] == 0
    assert st["maxInflight"] > 1, st  # the jobs overlapped on the device
    for (rc, I, info), ref, s in zip(out, alone, stream):
        assert rc in (0, 2)
        assert np.array_equal(I, np.triu(ref)), s.name
        assert info["units"] > 0 and info["msLatency"] >= info["msQueued"] >= 0 and info["msGpu"] > 0


def test_budget_admission(eg, stream):
    # a budget that holds about one of these jobs: they run one at a time
    one = max(eg_job_bytes(eg, s) for s in stream[:4])
    with eg.Server(mode=eg.ECPGB_FAST, budget_bytes=int(one * 1.5), slots=4) as sv:
        ids = [sv.submit(s) for s in stream[:4]]
        res = [sv.wait(i) for i in ids]
        st = sv.stats()
    assert st["completed"] == 4
    assert st["deviceBytesHeld"] <= int(one * 1.5)
    assert all(r[0] in (0, 2) for r in res)


def eg_job_bytes(eg, s):
    """Device bytes a served job held (read from a one-slot server)."""
    with eg.Server(mode=eg.ECPGB_FAST, budget_bytes=8 << 30, slots=1) as sv:
        return sv.wait(sv.submit(s))[2]["deviceBytes"]


def test_job_over_budget_fails_alone(eg, stream):
    big = W.batched_cluster(0)  # about 200 MB of device state
    with eg.Server(mode=eg.ECPGB_FAST, budget_bytes=32 << 20, slots=2) as sv:
        bad = sv.submit(big)
        ok = sv.submit(W.example_like(0))
        with pytest.raises(RuntimeError, match="budget"):
            sv.wait(bad)
        rc, I, _ = sv.wait(ok)
        st = sv.stats()
    ref = eg.get_integrals_info(W.example_like(0), mode=eg.ECPGB_FAST)[1]
    assert np.array_equal(I, np.triu(ref))
    assert st["failed"] == 1 and st["completed"] == 1


def test_poisson_stream_latency(eg):
    systems = serve.request_stream(30, seed=5, max_atoms=40, max_centres=10)
    arrivals = serve.poisson_arrivals(50.0, 30 / 50.0 * 1.2, seed=5)[:30]
    systems = systems[:len(arrivals)]
    with eg.Server(mode=eg.ECPGB_FAST, budget_bytes=4 << 30, slots=8) as sv:
        r = serve.run_stream(sv, systems, arrivals)
    assert r["requests"] == len(systems) and not r["errors"]
    lat = r["latency_ms"]
    assert 0 < lat["p50"] <= lat["p99"] <= lat["max"]


def test_small_request_overtakes_a_large_one(eg):
    """Continuous batching at unit granularity: a small request submitted
    right after a large one finishes first (the large job's CTAs take a few
    units each and the small job runs on a high-priority stream), and both
    results equal the same calls made alone."""
    big = W.batched_cluster(0)  # ~91k units, ~0.12 s of the whole GPU
    rng = np.random.default_rng(5)
    small = W.serving_molecule(rng, 6, 1)
    ref_big = eg.get_integrals_info(big, mode=eg.ECPGB_FAST)[1]
    ref_small = eg.get_integrals_info(small, mode=eg.ECPGB_FAST)[1]
    with eg.Server(mode=eg.ECPGB_FAST, budget_bytes=8 << 30, slots=4) as sv:
        sv.wait(sv.submit(big))  # warm: buffers, tables and schedules in place
        ib = sv.submit(big)
        isml = sv.submit(small)
        rs = sv.wait(isml)
        rb = sv.wait(ib)
    assert np.array_equal(rs[1], np.triu(ref_small)) and np.array_equal(rb[1], np.triu(ref_big))
    # the small request was done well inside the large one's run
    assert rs[2]["msLatency"] < 0.5 * rb[2]["msLatency"], (rs[2], rb[2])

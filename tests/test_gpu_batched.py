"""The batched engine's launch machinery: the persistent work-queue launch,
the cost-ordered queue, the captured CUDA graph and the autotuner.

queue / sorted / graph change only where and when units run, so the values
must agree bit for bit; gcap regroups the type-1 sums over warps (rounding
level), and every configuration stays within the parity bar of the FP64 path."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W
from tests.helpers import TOL_ABS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


@pytest.fixture(scope="module")
def system():
    return W.batched_cluster(0).subset(centres=list(range(6)))


def _run(eg, job, **cfg):
    if cfg:
        job.config(**cfg)
    job.run(1, flush_l2=False)
    return job.blocks()


def test_queue_order_and_graph_are_bitwise_neutral(eg, system):
    j = eg.Job(system, mode=eg.ECPGB_FAST)
    base_v, base_s = _run(eg, j, queue=1, sorted=1, gcap=45, screen=1)
    for cfg in ({"queue": 0, "sorted": 1}, {"queue": 0, "sorted": 0}, {"queue": 1, "sorted": 0},
                {"queue": 1, "sorted": 1, "screen": 0}, {"queue": 1, "sorted": 0, "screen": 1}):
        v, s = _run(eg, j, gcap=45, **cfg)
        assert np.array_equal(s, base_s), cfg
        assert np.array_equal(v, base_v), cfg
    j.config(queue=1, sorted=1, gcap=45, screen=1)
    j.use_graph(False)
    v, s = _run(eg, j)
    assert np.array_equal(v, base_v) and np.array_equal(s, base_s)
    j.use_graph(True)
    for _ in range(2):  # replays of one captured graph
        v, s = _run(eg, j)
        assert np.array_equal(v, base_v) and np.array_equal(s, base_s)
    j.close()


def test_every_config_within_parity_of_fp64(eg, system):
    jp = eg.Job(system, mode=eg.ECPGB_FP64)
    ref_v, ref_s = _run(eg, jp)
    jp.close()
    j = eg.Job(system, mode=eg.ECPGB_FAST)
    for gcap, balance in ((33, 1), (45, 1), (64, 1), (45, 0)):
        v, s = _run(eg, j, queue=1, sorted=1, gcap=gcap, balance=balance)
        assert np.array_equal(s, ref_s), gcap
        err = np.abs(v - ref_v).max()  # skipped units read zero in both
        assert err <= TOL_ABS, (gcap, err)
    j.close()


def test_autotuner_picks_a_measured_candidate(eg, system):
    j = eg.Job(system, mode=eg.ECPGB_FAST)
    chosen, trials = j.tune()
    assert len(trials) >= 4
    assert all(t["msUnit"] > 0 for t in trials)
    best = min(trials, key=lambda t: t["msUnit"])
    key = ("queue", "sorted", "gcap", "balance", "screen")
    assert tuple(chosen[k] for k in key) == tuple(best[k] for k in key)
    cur = j.config()
    assert tuple(cur[k] for k in key) == tuple(chosen[k] for k in key)
    # the tuned job still matches the drop-in matrix path
    ms, _ = j.run(1)
    I1 = j.matrix()
    rc, I2, _ = eg.get_integrals_info(system, mode=eg.ECPGB_FP64)
    assert np.abs(I1 - np.triu(I2)).max() <= TOL_ABS
    j.close()


def test_tuner_rejects_the_plain_path(eg, system):
    j = eg.Job(system, mode=eg.ECPGB_FP64)
    with pytest.raises(RuntimeError):
        j.tune()
    j.close()


def test_launches_per_run(eg, system):
    j = eg.Job(system, mode=eg.ECPGB_FAST)
    j.config(queue=1, screen=1)
    assert j.launches_per_run() == 10  # reset, 4 per-job stages, 3 screening, unit, scatter
    j.config(queue=0)
    assert j.launches_per_run() == 7
    j.close()


def test_screening_stage_marks_the_same_units(eg, system):
    jp = eg.Job(system, mode=eg.ECPGB_FP64)
    _, ref_s = _run(eg, jp)
    jp.close()
    j = eg.Job(system, mode=eg.ECPGB_FAST)
    _, s = _run(eg, j, queue=1, screen=1)
    assert np.array_equal(s, ref_s) and (s == 1).any() and (s != 1).any()
    j.close()


def test_per_class_settings_stay_within_parity(eg, system):
    """The autotuner's per-(la, lb) refinement: every class it sets has a cap
    within the launch's and a balance of 0 or 1, and the tuned job matches the
    FP64 path within the bar."""
    jp = eg.Job(system, mode=eg.ECPGB_FP64)
    ref_v, ref_s = _run(eg, jp)
    jp.close()
    j = eg.Job(system, mode=eg.ECPGB_FAST)
    chosen, trials = j.tune()
    cls = j.class_config()
    assert bool(cls) == bool(chosen["perClass"])
    for key, c in cls.items():
        assert 1 <= c["gcap"] <= chosen["gcap"] and c["balance"] in (0, 1), (key, c)
    assert any(t["perClass"] for t in trials) or chosen["queue"] != 1
    v, s = _run(eg, j)
    assert np.array_equal(s, ref_s)
    assert np.abs(v - ref_v).max() <= TOL_ABS
    j.close()

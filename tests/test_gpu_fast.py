"""Parity of the batched path (ECPGB_FAST) with the reference fixtures and the
oracle, at the same bar as the drop-in path: max abs error <= 1e-10."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import TOL_ABS, golden_files, load_golden, one_centre_answers, one_centre_system
from tests.test_gpu_parity import CASES, assert_blocks_match

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


@pytest.mark.parametrize("name", golden_files())
def test_fast_matches_reference_fixtures(eg, name):
    s, z = load_golden(name)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert_blocks_match(meta, data, z["meta"], z["data"])


@pytest.mark.parametrize("kw", CASES, ids=[f"seed{c['seed']}" for c in CASES])
def test_fast_matches_oracle(eg, kw):
    kw = dict(kw)
    s = W.random_system(kw.pop("seed"), **kw)
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert_blocks_match(meta, data, mo, do)


def test_fast_one_centre_known_answers(eg):
    s, _, _ = one_centre_system()
    rc, I, info = eg.get_integrals_info(s, mode=eg.ECPGB_FAST)
    for (i, j), v in one_centre_answers().items():
        assert abs(I[i, j] - v) <= 1e-12 * max(1.0, abs(v)), (i, j, I[i, j], v)


def test_fast_against_fp64_on_full_cluster(eg):
    """All 90k emitted units of the 50-centre cluster: batched vs drop-in path
    (the drop-in path is itself checked against the oracle)."""
    s = W.batched_cluster(0)
    m1, d1, st1, _ = eg.blocks(s, with_status=True)
    m2, d2, st2, _ = eg.blocks(s, mode=eg.ECPGB_FAST, with_status=True)
    assert np.array_equal(st1, st2)
    assert_blocks_match(m2, d2, m1, d1)


def test_fast_where_reference_aborts_and_forced_failures(eg):
    s = W.batched_cluster(0).subset(centres=[0], basis_atoms=[1, 6])
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert_blocks_match(meta, data, mo, do)
    s = W.random_system(26, n_atoms=2, n_centres=1, lmax_basis=1, lmax_ecp=2)
    s.tolerance = 1e-300
    rc, mo, do = O.oracle_blocks(s)
    meta, data, status, info = eg.blocks(s, mode=eg.ECPGB_FAST, with_status=True)
    assert info["firstFailed"] >= 0
    assert_blocks_match(meta, data, mo, do)


@pytest.mark.parametrize("order", [2048, 8190])
def test_fast_other_parameters(eg, order):
    """Large grids of 2047 and 4095 points, looser tolerance, other accuracy,
    non-integer r^n, contraction up to 8 (break searches over several
    chunks, the widest fallback bitmaps)."""
    s = W.random_system(23, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3, kmax=8)
    s.nECP[::3] += 0.5
    s.largeGridOrder, s.tolerance, s.accuracy = order, 1e-10, 1e-12
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert_blocks_match(meta, data, mo, do)


def test_fast_local_only_centre(eg):
    """A centre with only a local channel (the reference aborts on it): the
    type-1 part and a zero type-2 block, as the oracle."""
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=[(0, [(2.0, 2.0, 1.1)])], shells=[(1, [(0.7, 0.9)])])
    b.atom([0.5, -0.3, 0.8], shells=[(0, [(0.5, 0.4), (0.3, 2.0)]), (2, [(1.0, 0.6)])])
    s = b.build("local_only")
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert_blocks_match(meta, data, mo, do)


def test_fast_empty_inputs(eg):
    """No ECP centre: nothing is added, no block is emitted."""
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], shells=[(0, [(1.0, 1.0)])])
    s = b.build("no ecp")
    rc, I, _ = eg.get_integrals_info(s, mode=eg.ECPGB_FAST)
    assert rc == 0 and np.all(I == 0.0)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert meta.shape == (0, 8)


def test_fast_maximum_sizes(eg):
    rng = np.random.default_rng(5)
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=W._ecp_channels(rng, 5, 2), shells=[W._shell(rng, 4, 16, 0.05, 50.0)])
    b.atom([1.1, 0.4, -0.6], shells=[W._shell(rng, 4, 3, 0.05, 50.0), W._shell(rng, 0, 2, 0.1, 5)])
    s = b.build("max")
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s, mode=eg.ECPGB_FAST)
    assert_blocks_match(meta, data, mo, do)


def test_fast_job_deterministic(eg):
    s = W.random_system(27, n_atoms=4, n_centres=3, lmax_basis=3, lmax_ecp=3)
    job = eg.Job(s, mode=eg.ECPGB_FAST)
    job.run(1)
    I1 = job.matrix()
    job.run(1)
    I2 = job.matrix()
    job.close()
    assert np.array_equal(I1, I2)

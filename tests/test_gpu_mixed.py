"""The mixed-precision path (ECPGB_MIXED): the large-grid fallbacks' tables
(Bessel rows, ECP channels, powers of r, Gaussian prefactors) and integrand
products in double-single arithmetic on the FP32 pipes, level sums with a
compensated FP32 sum, everything else -- the small-grid quadratures, every
convergence test, every accumulation -- in FP64.

Bars: on the 50-centre cluster (s..f shells), max abs error <= 1e-10 against
the plain FP64 path on every unit and against the oracle.  Elsewhere (g
shells, large exponents) a block's rounding scales with its largest element
evaluated over absolute values (oracle_blocks_alt's scale, up to ~1e6 where
the shift onto A and B cancels), and double-single carries 2^-48 of it
where FP64 carries 2^-53: the bar is 1e-10 plus 2^-44 times the scale."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import TOL_ABS, bar_mixed, golden_files, load_golden
from tests.test_gpu_parity import CASES


def assert_mixed_match(s, meta, data):
    rc, mo, do, am, ad, sc = O.oracle_blocks_alt(s, 16.0)
    res = O.match_blocks(meta, data, mo, do, am, ad, bar_mixed, sc)
    assert not res["failures"], res["failures"][:5]


pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


@pytest.mark.parametrize("name", golden_files())
def test_mixed_matches_reference_fixtures(eg, name):
    s, z = load_golden(name)
    meta, data = eg.blocks(s, mode=eg.ECPGB_MIXED)
    assert np.array_equal(meta, z["meta"])
    assert_mixed_match(s, meta, data)


@pytest.mark.parametrize("kw", CASES, ids=[f"seed{c['seed']}" for c in CASES])
def test_mixed_matches_oracle(eg, kw):
    kw = dict(kw)
    s = W.random_system(kw.pop("seed"), **kw)
    meta, data = eg.blocks(s, mode=eg.ECPGB_MIXED)
    assert_mixed_match(s, meta, data)


def test_mixed_against_fp64_on_full_cluster(eg):
    """All 90k emitted units of the 50-centre cluster: the same statuses and
    blocks within 1e-10 of the plain FP64 path."""
    s = W.batched_cluster(0)
    v1, o1, st1, _ = eg.raw_blocks(s, eg.ECPGB_FP64)
    v3, o3, st3, _ = eg.raw_blocks(s, eg.ECPGB_MIXED)
    assert np.array_equal(st1, st3) and np.array_equal(o1, o3)
    assert np.isfinite(v3).all()
    err = float(np.max(np.abs(v3 - v1)))
    assert err <= TOL_ABS, err
    assert err > 0.0  # a different computation, not the FP64 one relabelled


def test_mixed_error_report_against_oracle(eg):
    """Per-(la, lb)-class max and rms error of the mixed path against the
    oracle (precision.class_errors) on three centres of the cluster."""
    from libecp_gb300.precision import oracle_class_errors
    s = W.batched_cluster(0)
    cs = [a for a in range(s.n_atoms) if s.shellsECP[a]]
    sub = s.subset(centres=cs[:3])
    rep = oracle_class_errors(sub, eg.ECPGB_MIXED)
    assert rep["classes"]["all"]["max_abs"] <= TOL_ABS, rep["classes"]["all"]
    for key, e in rep["classes"].items():
        assert set(e) == {"max_abs", "rms", "max_rel_block", "n_values", "n_units"}
        assert e["rms"] <= e["max_abs"]


@pytest.mark.parametrize("order", [2048, 8190])
def test_mixed_other_parameters(eg, order):
    """Large grids of 2047 and 4095 points, looser tolerance, other accuracy,
    non-integer r^n (the ECP powers outside 0, 1, 2 go through FP64)."""
    s = W.random_system(23, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3, kmax=8)
    s.nECP[::3] += 0.5
    s.largeGridOrder, s.tolerance, s.accuracy = order, 1e-10, 1e-12
    meta, data = eg.blocks(s, mode=eg.ECPGB_MIXED)
    assert_mixed_match(s, meta, data)


def test_mixed_where_reference_aborts_and_forced_failures(eg):
    s = W.batched_cluster(0).subset(centres=[0], basis_atoms=[1, 6])
    meta, data = eg.blocks(s, mode=eg.ECPGB_MIXED)
    assert_mixed_match(s, meta, data)
    s = W.random_system(26, n_atoms=2, n_centres=1, lmax_basis=1, lmax_ecp=2)
    s.tolerance = 1e-300
    meta, data, status, info = eg.blocks(s, mode=eg.ECPGB_MIXED, with_status=True)
    assert info["firstFailed"] >= 0
    assert_mixed_match(s, meta, data)


def test_mixed_matrix_and_job(eg):
    s = W.batched_cluster(0).subset(centres=[0, 1])
    rc, Imx, _ = eg.get_integrals_info(s, mode=eg.ECPGB_MIXED)
    j = eg.Job(s, mode=eg.ECPGB_MIXED)
    j.run(1)
    assert np.array_equal(j.matrix(), Imx)  # the job replays the same kernels
    j.run(1)
    assert np.array_equal(j.matrix(), Imx)  # and deterministically
    j.close()

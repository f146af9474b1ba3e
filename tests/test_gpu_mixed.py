"""The mixed-precision mode (ECPGB_MIXED): FP32 Bessel Taylor rows and ECP
channel terms, FP64 elsewhere, quadratures stopping at an FP32-consistent
relative floor.  It does not meet the FP64 bar and is not meant to: these
tests pin what it does deliver -- the per-L-class error report against the
FP64 path, errors at the 1e-3 level of the job's largest element in rms,
the same units emitted and nearly the same convergence statuses."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


@pytest.mark.parametrize("system", [W.example_like(0), W.batched_cluster(0).subset(centres=[0, 1, 2]),
                                    W.random_system(3, n_atoms=4, n_centres=2, lmax_basis=4, lmax_ecp=4)],
                         ids=["example", "cluster3", "g-shells"])
def test_mixed_error_report(eg, system):
    from libecp_gb300.precision import class_errors
    ref = eg.raw_blocks(system, eg.ECPGB_FP64)
    mx = eg.raw_blocks(system, eg.ECPGB_MIXED)
    rep = class_errors(system, ref, mx)
    allc = rep["classes"]["all"]
    scale = float(np.abs(ref[0]).max())
    assert allc["n_units"] == int(np.count_nonzero(ref[2] != 1))
    assert np.array_equal(ref[2] == 1, mx[2] == 1)  # the screening is FP64: same units
    assert np.count_nonzero(ref[2] != mx[2]) <= max(1, len(ref[2]) // 100)
    assert np.isfinite(mx[0]).all()
    assert allc["rms"] <= 1e-3 * scale, allc
    assert allc["max_abs"] > 0.0  # a different computation, not the FP64 one relabelled
    for key, e in rep["classes"].items():
        assert set(e) == {"max_abs", "rms", "max_rel_block", "n_values", "n_units"}


def test_mixed_matrix_and_job(eg):
    s = W.batched_cluster(0).subset(centres=[0, 1])
    rc, Imx, _ = eg.get_integrals_info(s, mode=eg.ECPGB_MIXED)
    j = eg.Job(s, mode=eg.ECPGB_MIXED)
    j.run(1)
    assert np.array_equal(j.matrix(), Imx)  # the job replays the same kernels
    j.close()

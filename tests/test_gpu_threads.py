"""Host threads: the engine serialises its device work behind one lock, so
concurrent calls from several threads (matrix, blocks, resident jobs, and
the request server's own worker) give each caller exactly what the call
gives alone."""
import threading

import numpy as np
import pytest

from libecp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


def test_concurrent_calls_match_serial(eg):
    systems = [W.random_system(40 + i, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3) for i in range(6)]
    modes = [eg.ECPGB_FP64, eg.ECPGB_FAST]
    alone = {(i, m): eg.get_integrals_info(s, mode=m)[1] for i, s in enumerate(systems) for m in modes}
    results, errors = {}, []

    def worker(k):
        try:
            for r in range(3):
                i = (k + r) % len(systems)
                m = modes[(k + r) % 2]
                results[(k, r)] = (i, m, eg.get_integrals_info(systems[i], mode=m)[1])
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))

    with eg.Server(mode=eg.ECPGB_FAST, budget_bytes=2 << 30, slots=4) as sv:
        ids = [sv.submit(s) for s in systems]  # the server's worker runs meanwhile
        threads = [threading.Thread(target=worker, args=(k,)) for k in range(6)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        served = [sv.wait(i)[1] for i in ids]
    assert not errors, errors
    for (i, m, I) in results.values():
        assert np.array_equal(I, alone[(i, m)])
    for i, I in enumerate(served):
        assert np.array_equal(I, np.triu(alone[(i, eg.ECPGB_FAST)]))

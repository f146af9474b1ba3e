"""Derivative fixtures and the shift semantics on the host (no GPU): the
recorded blocks follow the reference's shift table and skip rules
(src/libecp.c:240-330) and their sizes follow the block l of each shift
(src/libecp.c:356-362); where the reference build is present it reproduces
the fixtures bit for bit."""
import numpy as np
import pytest

from libecp_gb300 import SHIFTS, block_l
from libecp_gb300.workloads import ncart
from tests.helpers import deriv_golden_files, load_golden


@pytest.mark.parametrize("name", deriv_golden_files())
def test_shift_semantics(name):
    s, z = load_golden(name)
    n = s.derivative
    meta, data = z["meta"], z["data"]
    total = 0
    for A, s1, la, ha, B, s2, lb, hb, C, t in meta:
        assert (ha, hb) in SHIFTS[n]
        assert not (A == C and B == C)
        assert la + ha >= 0 and lb + hb >= 0
        if n == 1:
            assert not (C == A and ha != 0) and not (C == B and hb != 0)
        lpa, lpb = block_l(n, la, lb, ha, hb)
        total += ncart(lpa) * ncart(lpb)
    assert total == len(data)
    # per (pair, centre, shift): a type-1 then a type-2 block
    assert np.array_equal(meta[0::2, 9], np.ones(len(meta) // 2)) and np.all(meta[1::2, 9] == 2)


@pytest.mark.parametrize("name", deriv_golden_files())
def test_reference_reproduces_fixture(name):
    from oracle import oracle as O
    if not O.ref_available():
        pytest.skip("reference build not present on this machine")
    s, z = load_golden(name)
    rc, meta, data = O.ref_blocks_deriv(s, s.derivative)
    assert rc == 0
    assert np.array_equal(meta, z["meta"]) and np.array_equal(data, z["data"])


def test_ordered_fixture_reproduced_by_reference():
    from oracle import oracle as O
    from tests.helpers import ordered_golden_files
    if not O.ref_available():
        pytest.skip("reference build not present on this machine")
    for name in ordered_golden_files():
        s, z = load_golden(name)
        rc, meta, data = O.ref_blocks_ordered(s, s.ordering_lmax, s.ordering)
        assert rc == 0 and np.array_equal(meta, z["meta"]) and np.array_equal(data, z["data"])

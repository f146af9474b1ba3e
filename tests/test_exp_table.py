"""The committed exp table (libecp_gb300/csrc/ecp_exp2_table.h) is what its
generator writes: 2^(j/512) and the split ln2/512 from 256-bit arithmetic."""
import os
import subprocess
import sys

import pytest

from tests.helpers import ROOT

CSRC = os.path.join(ROOT, "libecp_gb300", "csrc")


def test_table_regenerates_identically(tmp_path):
    pytest.importorskip("mpmath")
    out = tmp_path / "table.h"
    subprocess.run([sys.executable, os.path.join(CSRC, "gen_exp2_table.py"), str(out)], check=True)
    with open(os.path.join(CSRC, "ecp_exp2_table.h")) as f:
        assert out.read_text() == f.read()


def test_table_values_round_to_nearest():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 256
    import re
    with open(os.path.join(CSRC, "ecp_exp2_table.h")) as f:
        text = f.read()
    vals = [float.fromhex(v) for v in re.findall(r"0x1\.[0-9a-f]+p[+-]0", text.split("ECPGB_EXP2_TABLE")[1])]
    assert len(vals) == 512
    for j in (0, 1, 17, 255, 256, 511):
        exact = mpmath.power(2, mpmath.mpf(j) / 512)
        err = abs(mpmath.mpf(vals[j]) - exact)
        ulp = mpmath.mpf(2) ** (math_floor_log2(vals[j]) - 52)
        assert err <= ulp / 2


def math_floor_log2(x):
    import math
    return math.frexp(x)[1] - 1

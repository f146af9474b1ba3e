"""The C-ABI library loads and exports every symbol include/*.h declares.
No compute calls (CPU only)."""
import ctypes as ct
import os
import re
import subprocess

import pytest

from tests.helpers import ROOT

LIB = os.path.join(ROOT, "libecp_gb300", "libecp_gb300.so")


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"typedef[^;]*;", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        subprocess.run(["python", "-m", "libecp_gb300.build"], cwd=ROOT, check=True)
    return ct.CDLL(LIB)


def test_headers_declare_the_dropin_interface():
    names = declared_functions()
    for n in ("getIntegrals", "libECP_init", "calculateECPIntegrals", "libECP_free", "newECP",
              "evalECP", "ECP_free", "ecpgb_blocks", "ecpgb_job_create", "ecpgb_measure_peaks"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ecp_helpers_host_only(lib):
    """newECP / evalECP / getECP / checkECP / ECP_free are host utilities."""
    class G(ct.Structure):
        _fields_ = [("l", ct.c_int), ("a", ct.c_double), ("d", ct.c_double), ("n", ct.c_double)]

    class E(ct.Structure):
        _fields_ = [("U_l", ct.POINTER(G)), ("N", ct.c_int), ("L", ct.c_int)]
    lib.newECP.restype = ct.POINTER(E)
    lib.evalECP.restype = ct.c_double
    lib.evalECP.argtypes = [ct.POINTER(E), ct.c_int, ct.c_double]
    e = lib.newECP(2, 3)
    terms = [(0, 1.3, 3.0, 2.0), (1, 0.7, -2.0, 2.0), (2, 2.1, 1.5, 1.0)]
    for i, (l, a, d, n) in enumerate(terms):
        e.contents.U_l[i] = G(l, a, d, n)
    r = 0.8
    assert abs(lib.evalECP(e, 1, r) - (-2.0 * r ** 2 * 2.718281828459045 ** (-0.7 * r * r))) < 1e-14
    assert lib.checkECP(e) == 0
    out = ct.POINTER(G)()
    assert lib.getECP(e, 2, ct.byref(out)) == 1 and abs(out[0].a - 2.1) < 1e-15
    lib.ECP_free(e)


def test_fails_loudly_without_gpu(lib):
    if os.path.exists("/dev/nvidia0") or os.path.exists("/dev/nvidiactl"):
        pytest.skip("a GPU is present: the no-GPU error path is not reachable")
    import numpy as np
    from libecp_gb300 import workloads as W
    import libecp_gb300 as eg
    s = W.example_like(0)
    with pytest.raises(RuntimeError, match="no CUDA device"):
        eg.get_integrals(s)
    I = np.zeros((s.dim, s.dim))
    assert not np.any(I)

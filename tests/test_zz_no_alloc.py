"""The entry point that allocates no device memory (ecpgb_getIntegrals_noalloc).

It serves host programs that keep all GPU memory in their own pool or arena,
or must not allocate inside a request: every device buffer comes from one
fixed array inside the library.  Through the C ABI, it must give the same
matrix as the ordinary getIntegrals on two calls in a row (the array keeps the
previous call's contents, so a second call -- and a call for another system
in between -- must not see leftovers), it must refuse a job too large for
the array with a clear error, and in a process where only it touches the GPU
the device's free memory must stay the same over calls for systems of
different sizes.  This file is collected last on purpose.
"""
import ctypes as ct
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from libecp_gb300 import workloads as W
from tests.helpers import ROOT, TOL_ABS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    L = libecp_gb300.lib()
    L.ecpgb_getIntegrals_noalloc.argtypes = [ct.POINTER(libecp_gb300.EcpgbSystem), ct.c_int,
                                             libecp_gb300._D]
    L.ecpgb_getIntegrals_noalloc.restype = ct.c_int
    L.ecpgb_noalloc_capacity.restype = ct.c_longlong
    return libecp_gb300


def noalloc(eg, s, I):
    cs = eg.c_system(s)
    return eg.lib().ecpgb_getIntegrals_noalloc(ct.byref(cs), I.shape[1], I.ctypes.data_as(eg._D))


def test_noalloc_matches_getintegrals_on_consecutive_calls(eg):
    a = W.example_like(0)
    b = W.random_system(40, n_atoms=4, n_centres=2, lmax_basis=3, lmax_ecp=4, kmax=3)
    ref = {id(a): eg.get_integrals(a), id(b): eg.get_integrals(b)}
    for s in (a, a, b, a):
        I = np.zeros((s.dim, s.dim))
        assert noalloc(eg, s, I) == 0, eg.last_error()
        assert np.max(np.abs(I - ref[id(s)])) <= TOL_ABS


def test_noalloc_accumulates_like_getintegrals(eg):
    s = W.random_system(41, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    rng = np.random.default_rng(3)
    I0 = rng.normal(size=(s.dim, s.dim + 3))
    I1, I2 = I0.copy(), I0.copy()
    assert eg.lib().getIntegrals(*eg._ptrs(s), I1.shape[1], I1.ctypes.data_as(eg._D)) == 0
    assert noalloc(eg, s, I2) == 0, eg.last_error()
    assert np.max(np.abs(I1 - I2)) <= TOL_ABS
    assert np.all(np.tril(I2[:, :s.dim] - I0[:, :s.dim], -1) == 0)


def test_noalloc_rejects_jobs_beyond_its_array(eg):
    s = W.batched_cluster(0)  # needs far more than the fixed array
    I = np.zeros((s.dim, s.dim))
    assert noalloc(eg, s, I) == 1
    assert "bytes of device scratch" in eg.last_error()
    assert not np.any(I)
    assert eg.lib().ecpgb_noalloc_capacity() == 64 << 20


# Child process: only the no-allocation entry point touches the GPU.  After
# one warm-up call (it creates the CUDA context and loads the module, with
# the scratch array, on the device), the device's free memory must not move
# over calls for systems of different sizes.
_FRESH = """
import ctypes as ct, json, sys
sys.path.insert(0, {root!r})
import numpy as np
import libecp_gb300 as eg
from libecp_gb300 import workloads as W
L = eg.lib()
L.ecpgb_getIntegrals_noalloc.argtypes = [ct.POINTER(eg.EcpgbSystem), ct.c_int, eg._D]
rt = ct.CDLL("libcudart.so.13")
def free_bytes():
    f, t = ct.c_size_t(0), ct.c_size_t(0)
    assert rt.cudaMemGetInfo(ct.byref(f), ct.byref(t)) == 0
    return f.value
def call(s):
    I = np.zeros((s.dim, s.dim))
    cs = eg.c_system(s)
    assert L.ecpgb_getIntegrals_noalloc(ct.byref(cs), s.dim, I.ctypes.data_as(eg._D)) == 0, eg.last_error()
    return I
systems = [W.example_like(0), W.random_system(40, n_atoms=4, n_centres=2, lmax_basis=3, lmax_ecp=4, kmax=3),
           W.batched_cluster(0).subset(centres=[0, 3], basis_atoms=range(4))]
first = call(systems[0])
f0 = free_bytes()
out = [call(s) for s in systems + systems]
f1 = free_bytes()
print(json.dumps({{"f0": f0, "f1": f1, "same": bool(np.array_equal(first, out[0]))}}))
"""


def test_noalloc_allocates_no_device_memory_in_a_fresh_process():
    code = _FRESH.format(root=ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       cwd=ROOT, env=dict(os.environ))
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["f0"] == res["f1"], res
    assert res["same"]

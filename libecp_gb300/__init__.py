"""libecp_gb300 -- GB300-native ECP integral engine behind libECP's C interface.

The product is the shared library ``libecp_gb300.so`` (CUDA kernels for
sm_103a plus the C ABI declared in ``include/``).  This module is a thin ctypes
view of that library for Python callers, tests and the benchmark; it performs
no arithmetic of its own, and it raises if the library has not been built --
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from .workloads import EcpSystem, ncart  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libecp_gb300.so")

_D = ct.POINTER(ct.c_double)
_I = ct.POINTER(ct.c_int)
_LL = ct.POINTER(ct.c_longlong)
_F = ct.POINTER(ct.c_float)

ECPGB_FP64 = 0   # plain FP64 kernels (the drop-in path)
ECPGB_FAST = 1   # batched FP64 path
ECPGB_MIXED = 2  # batched path with FP32 Bessel Taylor rows and ECP channel terms
UNIT_DONE, UNIT_SKIPPED, UNIT_WARN_TYPE1, UNIT_WARN_TYPE2 = 0, 1, 2, 3


class EcpgbSystem(ct.Structure):
    _fields_ = [("nrAtoms", ct.c_int), ("geometry", _D), ("shellsECP", _I), ("KECP", _I),
                ("lECP", _I), ("nECP", _D), ("dECP", _D), ("aECP", _D), ("shellsBS", _I),
                ("lBS", _I), ("KBS", _I), ("dBS", _D), ("aBS", _D), ("largeGridOrder", ct.c_int),
                ("tolerance", ct.c_double), ("accuracy", ct.c_double), ("derivative", ct.c_int),
                ("shellOrdering", _I), ("orderingLmax", ct.c_int)]


class EcpgbInfo(ct.Structure):
    _fields_ = [("units", ct.c_longlong), ("emitted", ct.c_longlong),
                ("firstFailed", ct.c_longlong), ("values", ct.c_longlong),
                ("msGpu", ct.c_double), ("msUnitKernel", ct.c_double),
                ("h2dBytes", ct.c_longlong), ("d2hBytes", ct.c_longlong)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class LaunchConfig(ct.Structure):
    """ecpgb_launch_config: batched-path launch configuration."""
    _fields_ = [("queue", ct.c_int), ("sorted", ct.c_int), ("gcap", ct.c_int), ("balance", ct.c_int),
                ("screen", ct.c_int), ("perClass", ct.c_int), ("msUnit", ct.c_float)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class RequestInfo(ct.Structure):
    """ecpgb_request_info: one served request."""
    _fields_ = [("units", ct.c_longlong), ("values", ct.c_longlong), ("msQueued", ct.c_double),
                ("msLatency", ct.c_double), ("msGpu", ct.c_double), ("deviceBytes", ct.c_longlong),
                ("slot", ct.c_int), ("firstFailed", ct.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class ServerStats(ct.Structure):
    """ecpgb_server_stats."""
    _fields_ = [("submitted", ct.c_longlong), ("completed", ct.c_longlong), ("failed", ct.c_longlong),
                ("queued", ct.c_longlong), ("inflight", ct.c_longlong), ("deviceBytesHeld", ct.c_longlong),
                ("budget", ct.c_longlong), ("slots", ct.c_int), ("maxInflight", ct.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


ECP_CALLBACK = ct.CFUNCTYPE(None, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
                            ct.c_int, ct.c_int, ct.c_int, _D, ct.c_void_p)

_lib = None


def lib() -> ct.CDLL:
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m libecp_gb300.build` "
            "(the ECP engine has no CPU fallback)")
    L = ct.CDLL(LIB_PATH)
    sys_args = [ct.c_int, _D, _I, _I, _I, _D, _D, _D, _I, _I, _I, _D, _D, ct.c_int, ct.c_double,
                ct.c_double]
    L.getIntegrals.argtypes = sys_args + [ct.c_int, _D]
    L.getIntegrals.restype = ct.c_int
    L.libECP_init.argtypes = [ct.c_int, _D, _I, _I, _I, _D, _D, _D, _I, _I, _I, _D, _D, ct.c_int,
                              ct.c_int, _I, ct.c_int, ct.c_double, ct.c_double]
    L.libECP_init.restype = ct.c_void_p
    L.calculateECPIntegrals.argtypes = [ct.c_void_p, ECP_CALLBACK, ct.c_void_p]
    L.calculateECPIntegrals.restype = ct.c_int
    L.libECP_free.argtypes = [ct.c_void_p]
    L.libECP_free.restype = None
    P = ct.POINTER(EcpgbSystem)
    L.ecpgb_layout.argtypes = [P, _LL, _LL]
    L.ecpgb_blocks.argtypes = [P, ct.c_int, _D, _LL, _I, ct.POINTER(EcpgbInfo)]
    L.ecpgb_getIntegrals.argtypes = [P, ct.c_int, ct.c_int, _D, ct.POINTER(EcpgbInfo)]
    L.ecpgb_job_create.argtypes = [P, ct.c_int]
    L.ecpgb_job_create.restype = ct.c_void_p
    L.ecpgb_job_run.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, _F, _F]
    L.ecpgb_job_matrix.argtypes = [ct.c_void_p, ct.c_int, _D]
    L.ecpgb_job_units.argtypes = [ct.c_void_p, _LL]
    L.ecpgb_job_units.restype = ct.c_longlong
    L.ecpgb_job_kernel_launches.argtypes = [ct.c_void_p]
    L.ecpgb_job_free.argtypes = [ct.c_void_p]
    L.ecpgb_job_tune.argtypes = [ct.c_void_p, ct.POINTER(LaunchConfig), ct.POINTER(LaunchConfig), ct.c_int,
                                 ct.POINTER(ct.c_int)]
    L.ecpgb_job_tune.restype = ct.c_int
    L.ecpgb_job_config.argtypes = [ct.c_void_p, ct.POINTER(LaunchConfig), ct.POINTER(LaunchConfig)]
    L.ecpgb_job_config.restype = ct.c_int
    L.ecpgb_job_class_config.argtypes = [ct.c_void_p, ct.c_int, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int)]
    L.ecpgb_job_class_config.restype = ct.c_int
    L.ecpgb_job_use_graph.argtypes = [ct.c_void_p, ct.c_int]
    L.ecpgb_job_use_graph.restype = ct.c_int
    L.ecpgb_job_blocks.argtypes = [ct.c_void_p, _D, _I]
    L.ecpgb_job_blocks.restype = ct.c_int
    L.ecpgb_server_create.argtypes = [ct.c_int, ct.c_longlong, ct.c_int]
    L.ecpgb_server_create.restype = ct.c_void_p
    L.ecpgb_server_submit.argtypes = [ct.c_void_p, P]
    L.ecpgb_server_submit.restype = ct.c_longlong
    L.ecpgb_server_poll.argtypes = [ct.c_void_p, ct.c_longlong]
    L.ecpgb_server_poll.restype = ct.c_int
    L.ecpgb_server_wait.argtypes = [ct.c_void_p, ct.c_longlong, ct.c_int, _D, ct.POINTER(RequestInfo)]
    L.ecpgb_server_wait.restype = ct.c_int
    L.ecpgb_server_get_stats.argtypes = [ct.c_void_p, ct.POINTER(ServerStats)]
    L.ecpgb_server_get_stats.restype = ct.c_int
    L.ecpgb_server_free.argtypes = [ct.c_void_p]
    L.ecpgb_server_free.restype = None
    L.ecpgb_layout_sph.argtypes = [P, _LL, _LL]
    L.ecpgb_layout_sph.restype = ct.c_int
    L.ecpgb_blocks_sph.argtypes = [P, ct.c_int, _D, _LL, _I]
    L.ecpgb_blocks_sph.restype = ct.c_int
    L.ecpgb_cart2sph.argtypes = [ct.c_int, _D]
    L.ecpgb_cart2sph.restype = ct.c_int
    L.ecpgb_gradient.argtypes = [P, ct.c_int, _D, ct.c_int, _D, _D]
    L.ecpgb_gradient.restype = ct.c_int
    L.ecpgb_load_system.argtypes = [ct.c_char_p, ct.c_char_p, ct.c_char_p]
    L.ecpgb_load_system.restype = ct.c_void_p
    L.ecpgb_loaded_system.argtypes = [ct.c_void_p]
    L.ecpgb_loaded_system.restype = ct.POINTER(EcpgbSystem)
    L.ecpgb_loaded_symbol.argtypes = [ct.c_void_p, ct.c_int]
    L.ecpgb_loaded_symbol.restype = ct.c_char_p
    L.ecpgb_loaded_free.argtypes = [ct.c_void_p]
    L.ecpgb_loaded_free.restype = None
    L.ecpgb_job_free.restype = None
    L.ecpgb_measure_peaks.argtypes = [_D]
    L.ecpgb_last_error.restype = ct.c_char_p
    L.ecpgb_set_device.argtypes = [ct.c_int]
    _lib = L
    return L


def last_error() -> str:
    return lib().ecpgb_last_error().decode()


def _ptrs(s: EcpSystem):
    d = lambda a: a.ctypes.data_as(_D)  # noqa: E731
    i = lambda a: a.ctypes.data_as(_I)  # noqa: E731
    return [s.n_atoms, d(s.geometry), i(s.shellsECP), i(s.KECP), i(s.lECP), d(s.nECP), d(s.dECP),
            d(s.aECP), i(s.shellsBS), i(s.lBS), i(s.KBS), d(s.dBS), d(s.aBS),
            int(s.largeGridOrder), float(s.tolerance), float(s.accuracy)]


def c_system(s: EcpSystem) -> EcpgbSystem:
    p = _ptrs(s)
    order = getattr(s, "ordering", None)
    if order is not None:
        order = np.ascontiguousarray(order, dtype=np.int32)
        s._ordering_c = order  # keep the buffer alive with the system
    return EcpgbSystem(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9], p[10], p[11],
                       p[12], p[13], p[14], p[15], int(getattr(s, "derivative", 0)),
                       order.ctypes.data_as(_I) if order is not None else None,
                       int(getattr(s, "ordering_lmax", 0)) if order is not None else 0)


def get_integrals(s: EcpSystem, I: np.ndarray | None = None) -> np.ndarray:
    """libECP's one-call interface: accumulates the upper triangle into I."""
    if I is None:
        I = np.zeros((s.dim, s.dim))
    rc = lib().getIntegrals(*_ptrs(s), I.shape[1], I.ctypes.data_as(_D))
    if rc != 0:
        raise RuntimeError(f"getIntegrals failed: {last_error()}")
    return I


def get_integrals_info(s: EcpSystem, mode: int = ECPGB_FP64):
    """(rc, matrix, info) through ecpgb_getIntegrals."""
    I = np.zeros((s.dim, s.dim))
    info = EcpgbInfo()
    cs = c_system(s)
    rc = lib().ecpgb_getIntegrals(ct.byref(cs), mode, s.dim, I.ctypes.data_as(_D), ct.byref(info))
    if rc == 1:
        raise RuntimeError(f"ecpgb_getIntegrals failed: {last_error()}")
    return rc, I, info.as_dict()


def raw_blocks(s: EcpSystem, mode: int = ECPGB_FP64):
    """ecpgb_blocks as arrays: (values, per-unit offsets, per-unit status, info)."""
    L = lib()
    cs = c_system(s)
    nu, nv = ct.c_longlong(0), ct.c_longlong(0)
    if L.ecpgb_layout(ct.byref(cs), ct.byref(nu), ct.byref(nv)):
        raise RuntimeError(last_error())
    vals = np.zeros(max(nv.value, 1))
    offs = np.zeros(max(nu.value, 1), dtype=np.int64)
    st = np.zeros(max(nu.value, 1), dtype=np.int32)
    info = EcpgbInfo()
    rc = L.ecpgb_blocks(ct.byref(cs), mode, vals.ctypes.data_as(_D), offs.ctypes.data_as(_LL),
                        st.ctypes.data_as(_I), ct.byref(info))
    if rc:
        raise RuntimeError(f"ecpgb_blocks failed: {last_error()}")
    return vals[:nv.value], offs[:nu.value], st[:nu.value], info.as_dict()


def blocks(s: EcpSystem, mode: int = ECPGB_FP64, with_status: bool = False):
    """All emitted blocks in the reference's callback order.

    Returns (meta, data) like the oracle: meta rows (A, s1, la, B, s2, lb, C,
    type), data the blocks back to back.
    """
    vals, offs, st, info = raw_blocks(s, mode)
    nu = ct.c_longlong(len(st))
    meta, data = [], []
    units = unit_table(s)
    for u in range(nu.value):
        if st[u] == UNIT_SKIPPED:
            continue
        A, s1, la, B, s2, lb, C = units[u]
        n = ncart(la) * ncart(lb)
        o = int(offs[u])
        meta.append((A, s1, la, B, s2, lb, C, 1))
        data.append(vals[o:o + n])
        meta.append((A, s1, la, B, s2, lb, C, 2))
        data.append(vals[o + n:o + 2 * n])
    meta = np.array(meta, dtype=np.int32).reshape(-1, 8)
    data = np.concatenate(data) if data else np.zeros(0)
    if with_status:
        return meta, data, st, info
    return meta, data


# Derivative shifts of libECP_init's order n (src/libecp.c:240-248).
SHIFTS = {0: [(0, 0)],
          1: [(1, 0), (-1, 0), (0, 1), (0, -1)],
          2: [(2, 0), (-2, 0), (1, 1), (1, -1), (-1, 1), (-1, -1), (0, 2), (0, -2), (1, 0), (0, 1)]}


def block_l(n: int, la: int, lb: int, ha: int, hb: int):
    """l of the blocks a shifted unit hands out (src/libecp.c:356-362)."""
    lpa, lpb = la + ha, lb + hb
    if n == 2 and (ha, hb) == (1, 0):
        lpa = la
    elif n == 2 and (ha, hb) == (0, 1):
        lpb = lb
    return lpa, lpb


def blocks_deriv(s: EcpSystem, mode: int = ECPGB_FP64, with_status: bool = False):
    """Derivative blocks (s.derivative = 1 or 2) in the reference's callback
    order: meta rows (A, s1, la, shifta, B, s2, lb, shiftb, C, type), data."""
    n = int(s.derivative)
    vals, offs, st, info = raw_blocks(s, mode)
    base = unit_table(s)  # (A, s1, la, B, s2, lb, C) per (centre, pair)
    shifts = SHIFTS[n]
    meta, data = [], []
    for i, (A, s1, la, B, s2, lb, C) in enumerate(base):
        for k, (ha, hb) in enumerate(shifts):
            u = i * len(shifts) + k
            if st[u] == UNIT_SKIPPED:
                continue
            lpa, lpb = block_l(n, la, lb, ha, hb)
            m = ncart(lpa) * ncart(lpb)
            o = int(offs[u])
            for t in (1, 2):
                meta.append((A, s1, la, ha, B, s2, lb, hb, C, t))
                data.append(vals[o + (t - 1) * m:o + t * m])
    meta = np.array(meta, dtype=np.int32).reshape(-1, 10)
    data = np.concatenate(data) if data else np.zeros(0)
    if with_status:
        return meta, data, st, info
    return meta, data


def unit_table(s: EcpSystem):
    """(A, s1, la, B, s2, lb, C) per unit u = centre_rank * nPairs + pair."""
    shells = []
    for a in range(s.n_atoms):
        for j in range(int(s.shellsBS[a])):
            shells.append((a, j))
    starts = np.concatenate([[0], np.cumsum(s.shellsBS)]).astype(int)
    pairs = []
    for A in range(s.n_atoms):
        for B in range(A, s.n_atoms):
            for i in range(int(s.shellsBS[A])):
                for j in range(int(s.shellsBS[B])):
                    if A == B and j < i:
                        continue
                    sa, sb = starts[A] + i, starts[B] + j
                    pairs.append((A, i, int(s.lBS[sa]), B, j, int(s.lBS[sb])))
    centres = [a for a in range(s.n_atoms) if s.shellsECP[a] > 0]
    return [p + (C,) for C in centres for p in pairs]


def calculate_blocks_via_callback(s: EcpSystem):
    """Drives libECP_init / calculateECPIntegrals / libECP_free and records the
    callback stream: (status, meta, data) in callback order.  Meta rows are
    (A, s1, la, B, s2, lb, C, type) for derivative order 0 and
    (A, s1, la, shifta, B, s2, lb, shiftb, C, type) otherwise."""
    L = lib()
    p = _ptrs(s)
    n = int(getattr(s, "derivative", 0))
    order = getattr(s, "ordering", None)
    lmax, optr = -1, None
    if order is not None:
        order = np.ascontiguousarray(order, dtype=np.int32)
        lmax, optr = int(s.ordering_lmax), order.ctypes.data_as(_I)
    # libECP_init reads (shellsECP, lECP, KECP) -- the definition's order
    h = L.libECP_init(p[0], p[1], p[2], p[4], p[3], p[5], p[6], p[7], p[8], p[9], p[10], p[11],
                      p[12], n, lmax, optr, p[13], p[14], p[15])
    if not h:
        raise RuntimeError(f"libECP_init failed: {last_error()}")
    meta, data = [], []
    last = {"key": None, "type": 0}

    def cb(A, sa, la, shifta, B, sb, lb, shiftb, C, I, _p):
        key = (A, sa, B, sb, C, shifta, shiftb)
        t = 2 if (last["key"] == key and last["type"] == 1) else 1
        last["key"], last["type"] = key, t
        lpa, lpb = block_l(n, la, lb, shifta, shiftb)
        m = ncart(lpa) * ncart(lpb)
        if n:
            meta.append((A, sa, la, shifta, B, sb, lb, shiftb, C, t))
        else:
            meta.append((A, sa, la, B, sb, lb, C, t))
        data.append(np.ctypeslib.as_array(I, shape=(m,)).copy())

    c_cb = ECP_CALLBACK(cb)
    try:
        rc = L.calculateECPIntegrals(h, c_cb, None)
    finally:
        L.libECP_free(h)
    meta = np.array(meta, dtype=np.int32).reshape(-1, 10 if n else 8)
    return rc, meta, (np.concatenate(data) if data else np.zeros(0))


class Job:
    """Device-resident job: inputs copied to HBM once, then re-run."""

    def __init__(self, s: EcpSystem, mode: int = ECPGB_FP64):
        self.system = s
        self._cs = c_system(s)
        self._h = lib().ecpgb_job_create(ct.byref(self._cs), mode)
        if not self._h:
            raise RuntimeError(f"ecpgb_job_create failed: {last_error()}")

    def run(self, n: int = 1, flush_l2: bool = True):
        ms = np.zeros(n, dtype=np.float32)
        mu = np.zeros(n, dtype=np.float32)
        if lib().ecpgb_job_run(self._h, n, int(flush_l2), ms.ctypes.data_as(_F),
                               mu.ctypes.data_as(_F)):
            raise RuntimeError(f"ecpgb_job_run failed: {last_error()}")
        return ms, mu

    def matrix(self) -> np.ndarray:
        I = np.zeros((self.system.dim, self.system.dim))
        if lib().ecpgb_job_matrix(self._h, self.system.dim, I.ctypes.data_as(_D)):
            raise RuntimeError(last_error())
        return I

    def units(self):
        em = ct.c_longlong(0)
        n = lib().ecpgb_job_units(self._h, ct.byref(em))
        return n, em.value

    def launches_per_run(self) -> int:
        return lib().ecpgb_job_kernel_launches(self._h)

    def tune(self):
        """Runs the autotuner; returns (chosen, trials) as dicts."""
        chosen = LaunchConfig()
        trials = (LaunchConfig * 32)()
        n = ct.c_int(0)
        rc = lib().ecpgb_job_tune(self._h, ct.byref(chosen), trials, 32, ct.byref(n))
        if rc:
            raise RuntimeError(f"ecpgb_job_tune failed ({rc}): {last_error()}")
        return chosen.as_dict(), [trials[i].as_dict() for i in range(n.value)]

    def config(self, queue=None, sorted=None, gcap=None, balance=None, screen=None) -> dict:
        """Reads the launch configuration; sets the fields given."""
        cur = LaunchConfig()
        if lib().ecpgb_job_config(self._h, None, ct.byref(cur)):
            raise RuntimeError(last_error())
        if all(v is None for v in (queue, sorted, gcap, balance, screen)):
            return cur.as_dict()
        new = LaunchConfig(cur.queue if queue is None else int(queue),
                           cur.sorted if sorted is None else int(sorted),
                           cur.gcap if gcap is None else int(gcap),
                           cur.balance if balance is None else int(balance),
                           cur.screen if screen is None else int(screen), 0, 0.0)
        if lib().ecpgb_job_config(self._h, ct.byref(new), ct.byref(cur)):
            raise RuntimeError(last_error())
        return cur.as_dict()

    def class_config(self) -> dict:
        """Per-(la, lb)-class type-1 settings of the configuration:
        {"la,lb": {"gcap": g, "balance": b}} for the classes the autotuner set."""
        n = 25
        g = (ct.c_int * n)()
        b = (ct.c_int * n)()
        if lib().ecpgb_job_class_config(self._h, n, g, b):
            raise RuntimeError(last_error())
        lb1 = self.system.max_l_basis() + 1 + getattr(self.system, "derivative", 0)
        out = {}
        for i in range(min(n, lb1 * lb1)):
            if g[i]:
                out[f"{i // lb1},{i % lb1}"] = {"gcap": int(g[i]), "balance": int(b[i])}
        return out

    def use_graph(self, on: bool = True) -> None:
        if lib().ecpgb_job_use_graph(self._h, int(on)):
            raise RuntimeError(last_error())

    def blocks(self):
        """Raw unit values (units' blocks at the ecpgb_blocks offsets) and the
        per-unit status of the last run."""
        cs = c_system(self.system)
        nu, nv = ct.c_longlong(0), ct.c_longlong(0)
        if lib().ecpgb_layout(ct.byref(cs), ct.byref(nu), ct.byref(nv)):
            raise RuntimeError(last_error())
        vals = np.zeros(max(nv.value, 1))
        st = np.zeros(max(nu.value, 1), dtype=np.int32)
        if lib().ecpgb_job_blocks(self._h, vals.ctypes.data_as(_D), st.ctypes.data_as(_I)):
            raise RuntimeError(last_error())
        return vals[:nv.value], st[:nu.value]

    def close(self):
        if self._h:
            lib().ecpgb_job_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_device(device: int) -> None:
    if lib().ecpgb_set_device(int(device)):
        raise RuntimeError(last_error())


def measure_peaks() -> dict:
    out = np.zeros(4)
    if lib().ecpgb_measure_peaks(out.ctypes.data_as(_D)):
        raise RuntimeError(last_error())
    return {"fp64_fma_tflops": out[0], "fp32_fma_tflops": out[1], "mufu_ex2_gops": out[2],
            "fp64_exp_gops": out[3]}


class Server:
    """Request server with continuous batching (ecpgb_server_*): jobs are
    admitted in arrival order as slots and device memory free up, and run on
    their own streams while earlier jobs are still on the GPU."""

    def __init__(self, mode: int = ECPGB_FAST, budget_bytes: int = 8 << 30, slots: int = 8):
        self._h = lib().ecpgb_server_create(mode, int(budget_bytes), int(slots))
        if not self._h:
            raise RuntimeError(f"ecpgb_server_create failed: {last_error()}")
        self._dims = {}

    def submit(self, s: EcpSystem) -> int:
        cs = c_system(s)
        rid = lib().ecpgb_server_submit(self._h, ct.byref(cs))
        if rid < 0:
            raise RuntimeError(f"ecpgb_server_submit failed: {last_error()}")
        self._dims[rid] = s.dim
        return rid

    def poll(self, rid: int) -> int:
        return lib().ecpgb_server_poll(self._h, rid)

    def wait(self, rid: int):
        """(rc, upper-triangle matrix, info dict); raises on failure."""
        dim = self._dims.pop(rid)
        I = np.zeros((dim, dim))
        info = RequestInfo()
        rc = lib().ecpgb_server_wait(self._h, rid, dim, I.ctypes.data_as(_D), ct.byref(info))
        if rc == 1:
            raise RuntimeError(f"request {rid} failed: {last_error()}")
        return rc, I, info.as_dict()

    def stats(self) -> dict:
        st = ServerStats()
        lib().ecpgb_server_get_stats(self._h, ct.byref(st))
        return st.as_dict()

    def close(self):
        if self._h:
            lib().ecpgb_server_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def libint_ordering(lmax: int) -> np.ndarray:
    """libint's Cartesian order of shells 0..lmax as exponent triples (the
    default order; a shellOrdering is a permutation within each shell)."""
    out = []
    for l in range(lmax + 1):
        for i in range(l + 1):
            for j in range(i + 1):
                out += [l - i, i - j, j]
    return np.array(out, dtype=np.int32)


def load_system(xyz: str, ecp: str, basis: str):
    """Reads the example program's text inputs (ecpgb_load_system): returns
    (EcpSystem, atom symbols).  No GPU needed."""
    L = lib()
    h = L.ecpgb_load_system(os.fsencode(xyz), os.fsencode(ecp), os.fsencode(basis))
    if not h:
        raise RuntimeError(f"ecpgb_load_system failed: {last_error()}")
    try:
        cs = L.ecpgb_loaded_system(h).contents
        n = cs.nrAtoms
        arr = lambda p, k, dt: np.ctypeslib.as_array(p, shape=(k,)).astype(dt).copy() if k else np.zeros(0, dt)
        shellsECP = arr(cs.shellsECP, n, np.int32)
        shellsBS = arr(cs.shellsBS, n, np.int32)
        nse, nsb = int(shellsECP.sum()), int(shellsBS.sum())
        KECP, lECP = arr(cs.KECP, nse, np.int32), arr(cs.lECP, nse, np.int32)
        KBS, lBS = arr(cs.KBS, nsb, np.int32), arr(cs.lBS, nsb, np.int32)
        nt, npr = int(KECP.sum()), int(KBS.sum())
        from .workloads import EcpSystem as _Sys
        s = _Sys(geometry=arr(cs.geometry, 3 * n, np.float64), shellsECP=shellsECP, KECP=KECP, lECP=lECP,
                 nECP=arr(cs.nECP, nt, np.float64), dECP=arr(cs.dECP, nt, np.float64),
                 aECP=arr(cs.aECP, nt, np.float64), shellsBS=shellsBS, lBS=lBS, KBS=KBS,
                 dBS=arr(cs.dBS, npr, np.float64), aBS=arr(cs.aBS, npr, np.float64),
                 largeGridOrder=cs.largeGridOrder, tolerance=cs.tolerance, accuracy=cs.accuracy,
                 name=os.path.basename(xyz))
        symbols = [L.ecpgb_loaded_symbol(h, i).decode() for i in range(n)]
    finally:
        L.ecpgb_loaded_free(h)
    return s, symbols


def gradient(s: EcpSystem, D: np.ndarray, mode: int = ECPGB_FP64):
    """(energy, gradient[nAtoms, 3]) of a symmetric density matrix D over the
    ECP matrix, both contracted on the GPU (ecpgb_gradient)."""
    D = np.ascontiguousarray(D, dtype=np.float64)
    assert D.shape == (s.dim, s.dim)
    cs = c_system(s)
    e = ct.c_double(0.0)
    g = np.zeros((s.n_atoms, 3))
    if lib().ecpgb_gradient(ct.byref(cs), mode, D.ctypes.data_as(_D), s.dim, ct.byref(e),
                            g.ctypes.data_as(_D)):
        raise RuntimeError(f"ecpgb_gradient failed: {last_error()}")
    return e.value, g


def cart2sph(l: int) -> np.ndarray:
    """The reference's Cartesian -> real spherical matrix T(l), (2l+1) x ncart(l)."""
    out = np.zeros((2 * l + 1, ncart(l)))
    if lib().ecpgb_cart2sph(int(l), out.ctypes.data_as(_D)):
        raise RuntimeError(last_error())
    return out


def blocks_sph(s: EcpSystem, mode: int = ECPGB_FP64):
    """Every emitted block in real spherical harmonics (ecpgb_blocks_sph), in
    the reference's callback order: (meta, data) as blocks() / blocks_deriv()."""
    L = lib()
    cs = c_system(s)
    nu, nv = ct.c_longlong(0), ct.c_longlong(0)
    if L.ecpgb_layout_sph(ct.byref(cs), ct.byref(nu), ct.byref(nv)):
        raise RuntimeError(last_error())
    vals = np.zeros(max(nv.value, 1))
    offs = np.zeros(max(nu.value, 1), dtype=np.int64)
    st = np.zeros(max(nu.value, 1), dtype=np.int32)
    if L.ecpgb_blocks_sph(ct.byref(cs), mode, vals.ctypes.data_as(_D), offs.ctypes.data_as(_LL),
                          st.ctypes.data_as(_I)):
        raise RuntimeError(f"ecpgb_blocks_sph failed: {last_error()}")
    n = int(getattr(s, "derivative", 0))
    shifts = SHIFTS[n]
    meta, data = [], []
    for i, (A, s1, la, B, s2, lb, C) in enumerate(unit_table(s)):
        for k, (ha, hb) in enumerate(shifts):
            u = i * len(shifts) + k
            if st[u] == UNIT_SKIPPED:
                continue
            lpa, lpb = block_l(n, la, lb, ha, hb)
            m = (2 * lpa + 1) * (2 * lpb + 1)
            o = int(offs[u])
            for t in (1, 2):
                meta.append((A, s1, la, ha, B, s2, lb, hb, C, t) if n else (A, s1, la, B, s2, lb, C, t))
                data.append(vals[o + (t - 1) * m:o + t * m])
    meta = np.array(meta, dtype=np.int32).reshape(-1, 10 if n else 8)
    return meta, (np.concatenate(data) if data else np.zeros(0))


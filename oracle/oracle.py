"""ctypes bindings for the parity checker -- TEST INFRASTRUCTURE ONLY.

* ``liboracle.so``: the CPU restatement in ecp_oracle.c (always available; built
  by ``make -C oracle``, which ``__graft_entry__.build()`` runs).
* ``_ref/libecp_ref.so``: the unmodified reference compiled by ``make -C oracle
  ref`` (only where the reference sources are present).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module.  Blocks come back in the reference's callback order with meta
rows (A, s1, la, B, s2, lb, C, type).
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libecp_ref.so")
REF_O0_SO = os.path.join(HERE, "_ref", "libecp_ref_O0.so")

_D = ct.POINTER(ct.c_double)
_I = ct.POINTER(ct.c_int)


class OracleStats(ct.Structure):
    _fields_ = [(n, ct.c_longlong) for n in (
        "blocks", "ps93_calls", "ps93_points", "ps93_failed", "psm92_calls", "psm92_points",
        "psm92_failed", "t1_prim_pairs", "t1_fallback_pp", "t2_items", "t2_fallback_items",
        "t2_fallback_pp", "bessel_calls", "bessel_rows", "exp_calls", "table_points",
        "contraction_fma", "stale_reads", "ps93_decisions", "ps93_divfree_flips")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


def _sys_argtypes():
    return [ct.c_int, _D, _I, _I, _I, _D, _D, _D, _I, _I, _I, _D, _D, ct.c_int, ct.c_double,
            ct.c_double]


def _sys_args(s):
    def d(a):
        return a.ctypes.data_as(_D)

    def i(a):
        return a.ctypes.data_as(_I)
    return [s.n_atoms, d(s.geometry), i(s.shellsECP), i(s.KECP), i(s.lECP), d(s.nECP),
            d(s.dECP), d(s.aECP), i(s.shellsBS), i(s.lBS), i(s.KBS), d(s.dBS), d(s.aBS),
            int(s.largeGridOrder), float(s.tolerance), float(s.accuracy)]


def build_oracle(force: bool = False) -> str:
    if force or not os.path.exists(ORACLE_SO) or \
            os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "ecp_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return ORACLE_SO


_oracle = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        lib = ct.CDLL(build_oracle())
        lib.oracle_blocks.argtypes = _sys_argtypes() + [ct.c_int, ct.c_int, ct.c_int, _I,
                                                        ct.c_longlong, _D, _I,
                                                        ct.POINTER(ct.c_longlong),
                                                        ct.POINTER(OracleStats)]
        lib.oracle_blocks_alt.argtypes = _sys_argtypes() + [ct.c_int, ct.c_int, ct.c_double, ct.c_int, _I,
                                                            ct.c_longlong, _D, _D, _I,
                                                            ct.POINTER(ct.c_longlong), ct.c_int, _I,
                                                            ct.c_longlong, _D, _I,
                                                            ct.POINTER(ct.c_longlong),
                                                            ct.POINTER(OracleStats)]
        lib.oracle_getIntegrals.argtypes = _sys_argtypes() + [ct.c_int, _D, ct.c_int, ct.c_int,
                                                              ct.POINTER(OracleStats)]
        lib.oracle_getIntegrals_mt.argtypes = _sys_argtypes() + [ct.c_int, _D, ct.c_int,
                                                                 ct.POINTER(OracleStats)]
        lib.oracle_grid.argtypes = [ct.c_int, ct.c_int, _D, _D]
        lib.oracle_bessel.argtypes = [ct.c_int, ct.c_double, ct.c_int, ct.c_double, _D]
        lib.oracle_rsh.argtypes = [ct.c_int, ct.c_double, ct.c_double, _D]
        _oracle = lib
    return _oracle


def _capacity(s, centres):
    from libecp_gb300.workloads import ncart
    nc = centres if centres is not None else max(s.n_centres, 1)
    per_pair = 0
    ls = [int(l) for l in s.lBS]
    n = len(ls)
    for i in range(n):
        for j in range(i, n):
            per_pair += ncart(ls[i]) * ncart(ls[j])
    return 2 * s.n_pairs * nc + 16, 2 * per_pair * nc + 16


def oracle_blocks(s, centre_lo=0, centre_hi=None, with_stats=False):
    """All blocks of the system (centres with index in [lo, hi))."""
    lib = oracle_lib()
    hi = s.n_atoms if centre_hi is None else centre_hi
    ncent = int(np.count_nonzero(s.shellsECP[centre_lo:hi]))
    mb, md = _capacity(s, ncent)
    meta = np.zeros(8 * mb, dtype=np.int32)
    data = np.zeros(md, dtype=np.float64)
    nb = ct.c_int(0)
    nd = ct.c_longlong(0)
    st = OracleStats()
    rc = lib.oracle_blocks(*_sys_args(s), centre_lo, hi, mb, meta.ctypes.data_as(_I), md,
                           data.ctypes.data_as(_D), ct.byref(nb), ct.byref(nd), ct.byref(st))
    meta = meta[:8 * nb.value].reshape(-1, 8).copy()
    data = data[:nd.value].copy()
    if with_stats:
        return rc, meta, data, st.as_dict()
    return rc, meta, data


def oracle_blocks_alt(s, kappa=16.0, centre_lo=0, centre_hi=None):
    """oracle_blocks plus the alternative blocks of decisions taken within
    rounding noise (see decide() in ecp_oracle.c): returns (rc, meta, data,
    alt_meta, alt_data, scale); alt rows carry the meta of the block they
    replace; scale[i] is block i's largest element evaluated over absolute
    values (its rounding-error scale)."""
    lib = oracle_lib()
    hi = s.n_atoms if centre_hi is None else centre_hi
    ncent = int(np.count_nonzero(s.shellsECP[centre_lo:hi]))
    mb, md = _capacity(s, ncent)
    meta = np.zeros(8 * mb, dtype=np.int32)
    data = np.zeros(md, dtype=np.float64)
    scale = np.zeros(mb, dtype=np.float64)
    for grow in (2, 20):  # alternatives per block: up to 19 (see run_centre)
        ma, mda = grow * mb + 64, grow * md + 4096
        ameta = np.zeros(8 * ma, dtype=np.int32)
        adata = np.zeros(mda, dtype=np.float64)
        nb, na = ct.c_int(0), ct.c_int(0)
        nd, nad = ct.c_longlong(0), ct.c_longlong(0)
        st = OracleStats()
        rc = lib.oracle_blocks_alt(*_sys_args(s), centre_lo, hi, float(kappa), mb, meta.ctypes.data_as(_I),
                                   md, data.ctypes.data_as(_D), scale.ctypes.data_as(_D), ct.byref(nb),
                                   ct.byref(nd), ma,
                                   ameta.ctypes.data_as(_I), mda, adata.ctypes.data_as(_D), ct.byref(na),
                                   ct.byref(nad), ct.byref(st))
        if rc != -2:
            break
    return (rc, meta[:8 * nb.value].reshape(-1, 8).copy(), data[:nd.value].copy(),
            ameta[:8 * na.value].reshape(-1, 8).copy(), adata[:nad.value].copy(), scale[:nb.value].copy())


def match_blocks(meta, data, ref_meta, ref_data, alt_meta=None, alt_data=None, bar=None, scale=None):
    """Compares blocks in callback order against the reference blocks.

    A block passes when its largest element difference from the reference
    block is within bar(block), or from one of the block's alternatives (the
    reference's results with a decision taken within rounding noise
    inverted).  bar(ref_block) -> allowed absolute difference, or
    bar(ref_block, scale_i) when the blocks' scales are given.  Returns a
    dict: n_blocks, n_alt_used, worst (largest diff / bar over the passing
    choice), failures (list of (meta row, diff, bar)), max_abs."""
    assert np.array_equal(meta, ref_meta), "block lists differ"
    alts = {}
    if alt_meta is not None:
        off = 0
        for m in alt_meta:
            n = ((m[2] + 1) * (m[2] + 2) // 2) * ((m[5] + 1) * (m[5] + 2) // 2)
            alts.setdefault(tuple(int(x) for x in m), []).append(alt_data[off:off + n])
            off += n
    out = {"n_blocks": len(meta), "n_alt_used": 0, "worst": 0.0, "failures": [], "max_abs": 0.0}
    off = 0
    for i, m in enumerate(meta):
        n = ((m[2] + 1) * (m[2] + 2) // 2) * ((m[5] + 1) * (m[5] + 2) // 2)
        g, r = data[off:off + n], ref_data[off:off + n]
        off += n
        b = bar(r) if scale is None else bar(r, scale[i])
        d = float(np.max(np.abs(g - r))) if n else 0.0
        if d > b:
            for a in alts.get(tuple(int(x) for x in m), []):
                da = float(np.max(np.abs(g - a)))
                if da <= b:
                    out["n_alt_used"] += 1
                    d = da
                    break
        if d > b:
            out["failures"].append((tuple(int(x) for x in m), d, b))
        out["worst"] = max(out["worst"], d / b)
        out["max_abs"] = max(out["max_abs"], d)
    return out


def oracle_matrix(s, nthreads=1, with_stats=False):
    lib = oracle_lib()
    dim = s.dim
    I = np.zeros((dim, dim), dtype=np.float64)
    st = OracleStats()
    if nthreads <= 1:
        rc = lib.oracle_getIntegrals(*_sys_args(s), dim, I.ctypes.data_as(_D), 0, s.n_atoms,
                                     ct.byref(st))
    else:
        rc = lib.oracle_getIntegrals_mt(*_sys_args(s), dim, I.ctypes.data_as(_D), nthreads,
                                        ct.byref(st))
    if with_stats:
        return rc, I, st.as_dict()
    return rc, I


# --------------------------------------------------------------- reference

def ref_available(path=REF_SO) -> bool:
    if not os.path.exists(path):
        return False
    try:
        ct.CDLL(path)
        return True
    except OSError:  # e.g. built for another architecture
        return False


_ref = {}


def ref_lib(path=REF_SO):
    if path not in _ref:
        lib = ct.CDLL(path)
        lib.ref_blocks.argtypes = _sys_argtypes() + [ct.c_int, _I, ct.c_longlong, _D, _I,
                                                     ct.POINTER(ct.c_longlong)]
        lib.getIntegrals.argtypes = _sys_argtypes() + [ct.c_int, _D]
        lib.getIntegrals.restype = ct.c_int
        lib.ref_blocks_deriv.argtypes = _sys_argtypes() + [ct.c_int, ct.c_int, _I, ct.c_longlong, _D, _I,
                                                           ct.POINTER(ct.c_longlong)]
        lib.ref_blocks_ordered.argtypes = _sys_argtypes() + [ct.c_int, _I, ct.c_int, _I, ct.c_longlong, _D,
                                                             _I, ct.POINTER(ct.c_longlong)]
        _ref[path] = lib
    return _ref[path]


def ref_blocks(s, path=REF_SO):
    """All blocks the unmodified reference hands to its callback."""
    lib = ref_lib(path)
    mb, md = _capacity(s, None)
    meta = np.zeros(8 * mb, dtype=np.int32)
    data = np.zeros(md, dtype=np.float64)
    nb = ct.c_int(0)
    nd = ct.c_longlong(0)
    rc = lib.ref_blocks(*_sys_args(s), mb, meta.ctypes.data_as(_I), md, data.ctypes.data_as(_D),
                        ct.byref(nb), ct.byref(nd))
    return rc, meta[:8 * nb.value].reshape(-1, 8).copy(), data[:nd.value].copy()


def ref_blocks_deriv(s, n, path=REF_SO):
    """The reference's derivative blocks (libECP_init with derivative order n):
    meta rows (A, s1, la, shifta, B, s2, lb, shiftb, C, type) and the data."""
    lib = ref_lib(path)
    mb, md = _capacity(s, None)
    mb, md = 10 * mb, 80 * md  # up to 10 shifts, blocks of l + 2
    meta = np.zeros(10 * mb, dtype=np.int32)
    data = np.zeros(md, dtype=np.float64)
    nb = ct.c_int(0)
    nd = ct.c_longlong(0)
    rc = lib.ref_blocks_deriv(*_sys_args(s), int(n), mb, meta.ctypes.data_as(_I), md,
                              data.ctypes.data_as(_D), ct.byref(nb), ct.byref(nd))
    return rc, meta[:10 * nb.value].reshape(-1, 10).copy(), data[:nd.value].copy()


def ref_blocks_ordered(s, lmax, ordering, path=REF_SO):
    """The reference's blocks in a caller's Cartesian order (libECP_init's
    lmax and shellOrdering)."""
    lib = ref_lib(path)
    mb, md = _capacity(s, None)
    meta = np.zeros(8 * mb, dtype=np.int32)
    data = np.zeros(md, dtype=np.float64)
    order = np.ascontiguousarray(ordering, dtype=np.int32)
    nb = ct.c_int(0)
    nd = ct.c_longlong(0)
    rc = lib.ref_blocks_ordered(*_sys_args(s), int(lmax), order.ctypes.data_as(_I), mb,
                                meta.ctypes.data_as(_I), md, data.ctypes.data_as(_D), ct.byref(nb),
                                ct.byref(nd))
    return rc, meta[:8 * nb.value].reshape(-1, 8).copy(), data[:nd.value].copy()


def ref_matrix(s, path=REF_SO):
    lib = ref_lib(path)
    dim = s.dim
    I = np.zeros((dim, dim), dtype=np.float64)
    rc = lib.getIntegrals(*_sys_args(s), dim, I.ctypes.data_as(_D))
    return rc, I


def split_blocks(meta, data):
    """List of (key, block) with key = (C, A, s1, B, s2, type)."""
    out = []
    off = 0
    for m in meta:
        na = (m[2] + 1) * (m[2] + 2) // 2
        nb = (m[5] + 1) * (m[5] + 2) // 2
        out.append(((int(m[6]), int(m[0]), int(m[1]), int(m[3]), int(m[4]), int(m[7])),
                    data[off:off + na * nb].reshape(na, nb)))
        off += na * nb
    return out

"""Generates the golden fixtures in this folder from the unmodified reference.

Run where the reference sources are present (they are compiled by
``make -C oracle ref`` into oracle/_ref/libecp_ref.so, -O2, no fast-math):

    python tests/golden/make_golden.py

Each fixture is a compressed .npz holding one seeded system (the
getIntegrals arrays) and every block the reference handed to its callback,
in callback order: meta rows (A, s1, la, B, s2, lb, C, type) and the blocks
back to back.  Systems whose basis l reaches the ECP's L are run on the
reference with a zero-coefficient high-l pad centre (EcpSystem.padded), which
keeps the reference's table reads in bounds and adds exactly zero; the blocks
are those of the unpadded system.  The example-like fixture also stores the
reference's getIntegrals matrix.

The ordered_* fixtures hold blocks in a caller's Cartesian order
(libECP_init's lmax and shellOrdering; here libint's order reversed within
each shell).  The deriv*_ fixtures hold the nuclear-derivative blocks of libECP_init's
order n (1 or 2): meta rows (A, s1, la, shifta, B, s2, lb, shiftb, C, type).
Their systems keep basis l + n below the ECP's L, where the reference's
tables stay in bounds without padding.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libecp_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    "example_like_s0": lambda: W.example_like(0),
    "random_s0": lambda: W.random_system(0, n_atoms=4, n_centres=2, lmax_basis=2, lmax_ecp=3),
    "random_s1": lambda: W.random_system(1, n_atoms=4, n_centres=2, lmax_basis=2, lmax_ecp=3),
    "random_g_s101": lambda: W.random_system(101, n_atoms=3, n_centres=2, lmax_basis=4,
                                             lmax_ecp=3, kmax=2),
    "random_fL5_s200": lambda: W.random_system(200, n_atoms=3, n_centres=2, lmax_basis=3,
                                               lmax_ecp=5, kmax=3, elo=0.01, ehi=500),
    "cluster_subset_s0": lambda: W.batched_cluster(0).subset(centres=[0, 1],
                                                             basis_atoms=range(6)),
}


DERIV_CASES = {
    "deriv1_s3": (1, lambda: W.random_system(3, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=4)),
    "deriv1_s6": (1, lambda: W.random_system(6, n_atoms=4, n_centres=2, lmax_basis=1, lmax_ecp=3, kmax=3)),
    "deriv2_s4": (2, lambda: W.random_system(4, n_atoms=3, n_centres=2, lmax_basis=1, lmax_ecp=4)),
    "deriv2_s5": (2, lambda: W.random_system(5, n_atoms=3, n_centres=1, lmax_basis=2, lmax_ecp=5, kmax=2)),
}


def reversed_ordering(lmax):
    """libint's Cartesian order with every shell reversed."""
    from libecp_gb300 import libint_ordering
    from libecp_gb300.workloads import ncart
    d = libint_ordering(lmax)
    out, off = [], 0
    for l in range(lmax + 1):
        out.append(d[off:off + 3 * ncart(l)].reshape(-1, 3)[::-1].ravel())
        off += 3 * ncart(l)
    return np.concatenate(out).astype(np.int32)


# blocks in a caller's Cartesian order (libECP_init's lmax, shellOrdering)
ORDERED_CASES = {
    "ordered_rev_s2": lambda: W.random_system(2, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3),
}


def save_ordered(name, s):
    lmax = s.max_l_ecp() + 2 * s.max_l_basis()
    order = reversed_ordering(lmax)
    rc, meta, data = O.ref_blocks_ordered(s, lmax, order)
    if rc != 0:
        raise RuntimeError(f"reference failed on {name}: {rc}")
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), geometry=s.geometry, shellsECP=s.shellsECP,
        KECP=s.KECP, lECP=s.lECP, nECP=s.nECP, dECP=s.dECP, aECP=s.aECP, shellsBS=s.shellsBS,
        lBS=s.lBS, KBS=s.KBS, dBS=s.dBS, aBS=s.aBS,
        params=np.array([s.largeGridOrder, s.tolerance, s.accuracy]), ordering=order,
        ordering_lmax=np.array(lmax), padded=np.array(False), meta=meta, data=data)
    print(f"{name}: ordering lmax={lmax}, {len(meta)} blocks, max|I|={np.abs(data).max():.3e}")


def save_deriv(name, n, s):
    assert s.max_l_basis() + n < s.max_l_ecp()
    rc, meta, data = O.ref_blocks_deriv(s, n)
    if rc != 0:
        raise RuntimeError(f"reference failed on {name}: {rc}")
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), geometry=s.geometry, shellsECP=s.shellsECP,
        KECP=s.KECP, lECP=s.lECP, nECP=s.nECP, dECP=s.dECP, aECP=s.aECP, shellsBS=s.shellsBS,
        lBS=s.lBS, KBS=s.KBS, dBS=s.dBS, aBS=s.aBS,
        params=np.array([s.largeGridOrder, s.tolerance, s.accuracy]), derivative=np.array(n),
        padded=np.array(False), meta=meta, data=data)
    print(f"{name}: n={n}, {len(meta)} blocks, max|I|={np.abs(data).max():.3e}")


def save(name, s):
    sr = s.padded() if s.needs_pad() else s
    rc, meta, data = O.ref_blocks(sr)
    if rc != 0:
        raise RuntimeError(f"reference failed on {name}: {rc}")
    extra = {}
    if name.startswith("example_like"):
        rcm, I = O.ref_matrix(sr)
        extra["matrix"] = I
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), geometry=s.geometry, shellsECP=s.shellsECP,
        KECP=s.KECP, lECP=s.lECP, nECP=s.nECP, dECP=s.dECP, aECP=s.aECP, shellsBS=s.shellsBS,
        lBS=s.lBS, KBS=s.KBS, dBS=s.dBS, aBS=s.aBS,
        params=np.array([s.largeGridOrder, s.tolerance, s.accuracy]),
        padded=np.array(sr is not s), meta=meta, data=data, **extra)
    print(f"{name}: {len(meta)} blocks, padded={sr is not s}, max|I|={np.abs(data).max():.3e}")


def load(path) -> tuple:
    z = np.load(path)
    p = z["params"]
    s = W.EcpSystem(z["geometry"], z["shellsECP"], z["KECP"], z["lECP"], z["nECP"], z["dECP"],
                    z["aECP"], z["shellsBS"], z["lBS"], z["KBS"], z["dBS"], z["aBS"],
                    int(p[0]), float(p[1]), float(p[2]), name=os.path.basename(path),
                    derivative=int(z["derivative"]) if "derivative" in z.files else 0)
    if "ordering" in z.files:
        s.ordering = z["ordering"]
        s.ordering_lmax = int(z["ordering_lmax"])
    return s, z


if __name__ == "__main__":
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    for name, make in CASES.items():
        save(name, make())
    for name, (n, make) in DERIV_CASES.items():
        save_deriv(name, n, make())
    for name, make in ORDERED_CASES.items():
        save_ordered(name, make())
    with open(os.path.join(HERE, "PROVENANCE.txt"), "w") as f:
        gcc = subprocess.run(["gcc", "--version"], capture_output=True, text=True).stdout.splitlines()[0]
        libc = " ".join(platform.libc_ver())
        f.write("Produced by tests/golden/make_golden.py from the unmodified chrr/libECP sources\n"
                f"compiled with `gcc -O2 -fPIC` ({gcc}, {libc}, {platform.machine()}).\n")

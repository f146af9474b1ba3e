"""Seeded synthetic ECP systems.

An :class:`EcpSystem` carries exactly the arrays libECP's one-call interface
takes (``getIntegrals``, src/getIntegrals.h:7-13 of chrr/libECP):

* ``geometry[3*nAtoms]`` in bohr;
* ``shellsECP[nAtoms]`` ECP shells per atom (0 = no ECP on that atom);
* ``KECP`` (terms per ECP shell) and ``lECP`` (l of each ECP shell);
* ``nECP, dECP, aECP`` one entry per ECP term: U(r) = d r^n exp(-a r^2);
* ``shellsBS[nAtoms]`` basis shells per atom, ``lBS``/``KBS`` per shell;
* ``dBS, aBS`` per primitive (coefficients are used raw, as the reference does).

The generators draw every quantity from ``numpy.random.default_rng(seed)`` in
a fixed, documented order, so the same seed gives the same system on every
machine.  No public data set is involved: these are the synthetic stand-ins
for the benchmark configurations (single-centre example-like system, batched
cluster, mixed-precision batch, serving stream, large high-accuracy sweep).
"""
from __future__ import annotations

from dataclasses import dataclass, field
import numpy as np


def ncart(l: int) -> int:
    """Number of Cartesian functions of a shell (IJK_DIM, src/dimensions.h:36)."""
    return (l + 1) * (l + 2) // 2


@dataclass
class EcpSystem:
    geometry: np.ndarray
    shellsECP: np.ndarray
    KECP: np.ndarray
    lECP: np.ndarray
    nECP: np.ndarray
    dECP: np.ndarray
    aECP: np.ndarray
    shellsBS: np.ndarray
    lBS: np.ndarray
    KBS: np.ndarray
    dBS: np.ndarray
    aBS: np.ndarray
    largeGridOrder: int = 1024
    tolerance: float = 1.0e-12
    accuracy: float = 1.0e-14
    name: str = field(default="system")
    # nuclear-derivative order of libECP_init (0, 1, 2): blocks of shifted shells
    derivative: int = 0
    # libECP_init's shellOrdering: Cartesian exponent triples of shells
    # l = 0..ordering_lmax in the caller's order (None: libint's)
    ordering: np.ndarray | None = None
    ordering_lmax: int = 0

    def __post_init__(self):
        self.geometry = np.ascontiguousarray(self.geometry, dtype=np.float64).reshape(-1)
        for k in ("shellsECP", "KECP", "lECP", "shellsBS", "lBS", "KBS"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32).reshape(-1))
        for k in ("nECP", "dECP", "aECP", "dBS", "aBS"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64).reshape(-1))

    # ------------------------------------------------------------------ sizes
    @property
    def n_atoms(self) -> int:
        return int(self.shellsBS.shape[0])

    @property
    def n_shells(self) -> int:
        return int(self.lBS.shape[0])

    @property
    def dim(self) -> int:
        """AO dimension (sum of Cartesian shell sizes)."""
        return int(sum(ncart(int(l)) for l in self.lBS))

    @property
    def n_centres(self) -> int:
        return int(np.count_nonzero(self.shellsECP))

    @property
    def n_pairs(self) -> int:
        """Shell pairs the reference visits: every (A<=B, s1, s2) with s2>=s1 when A==B."""
        n = self.n_shells
        return n * (n + 1) // 2

    @property
    def n_units(self) -> int:
        """(shell pair, ECP centre) units before screening."""
        return self.n_pairs * self.n_centres

    def max_l_basis(self) -> int:
        return int(self.lBS.max()) if self.n_shells else 0

    def max_l_ecp(self) -> int:
        return int(self.lECP.max()) if self.lECP.size else 0

    def args(self):
        """Arguments in getIntegrals order (without rowdim / I)."""
        return (self.n_atoms, self.geometry, self.shellsECP, self.KECP, self.lECP,
                self.nECP, self.dECP, self.aECP, self.shellsBS, self.lBS, self.KBS,
                self.dBS, self.aBS, self.largeGridOrder, self.tolerance, self.accuracy)

    def needs_pad(self) -> bool:
        """True when the reference would read past its potential table.

        The reference sizes its r^k U_l table by maxLambda = maxL_ECP - 1 +
        maxL_basis (src/type2.c:185-219 via :51-54) but reads rows up to
        la + lb (src/type2.c:364); that overruns when maxL_basis >= maxL_ECP.
        Its Bessel table needs maxL_basis <= maxL_ECP + 1 (src/bessel.c:137-151).
        """
        lb, le = self.max_l_basis(), self.max_l_ecp()
        return 2 * lb > le - 1 + lb or lb > le + 1

    def padded(self, pad_l: int | None = None) -> "EcpSystem":
        """Adds a basis-less atom carrying one zero-coefficient ECP term of high l.

        That raises the reference's global table sizes so every read is in
        bounds while adding exactly zero to every integral (the pad centre's
        channels all vanish, so its screening skips every shell).  Used only
        to drive the reference; the engine computes the in-bounds values
        directly.
        """
        if pad_l is None:
            pad_l = max(self.max_l_basis() + 1, self.max_l_ecp()) + 1
        far = np.array([0.0, 0.0, 0.0])
        return EcpSystem(
            geometry=np.concatenate([self.geometry, far]),
            shellsECP=np.concatenate([self.shellsECP, [1]]),
            KECP=np.concatenate([self.KECP, [1]]),
            lECP=np.concatenate([self.lECP, [pad_l]]),
            nECP=np.concatenate([self.nECP, [0.0]]),
            dECP=np.concatenate([self.dECP, [0.0]]),
            aECP=np.concatenate([self.aECP, [1.0]]),
            shellsBS=np.concatenate([self.shellsBS, [0]]),
            lBS=self.lBS.copy(), KBS=self.KBS.copy(), dBS=self.dBS.copy(), aBS=self.aBS.copy(),
            largeGridOrder=self.largeGridOrder, tolerance=self.tolerance,
            accuracy=self.accuracy, name=self.name + "+pad")

    def subset(self, centres=None, basis_atoms=None) -> "EcpSystem":
        """Same geometry; keeps the ECPs of `centres` and the basis of `basis_atoms`."""
        na = self.n_atoms
        centres = range(na) if centres is None else set(int(c) for c in centres)
        basis_atoms = range(na) if basis_atoms is None else set(int(a) for a in basis_atoms)
        sE, K, lE, nE, dE, aE = [], [], [], [], [], []
        sB, lB, KB, dB, aB = [], [], [], [], []
        ie = it = ib = ip = 0
        for a in range(na):
            ne = int(self.shellsECP[a])
            keep = a in centres
            sE.append(ne if keep else 0)
            for _ in range(ne):
                k = int(self.KECP[ie])
                if keep:
                    K.append(k); lE.append(int(self.lECP[ie]))
                    nE += list(self.nECP[it:it + k]); dE += list(self.dECP[it:it + k])
                    aE += list(self.aECP[it:it + k])
                ie += 1
                it += k
            nb = int(self.shellsBS[a])
            keepb = a in basis_atoms
            sB.append(nb if keepb else 0)
            for _ in range(nb):
                k = int(self.KBS[ib])
                if keepb:
                    lB.append(int(self.lBS[ib])); KB.append(k)
                    dB += list(self.dBS[ip:ip + k]); aB += list(self.aBS[ip:ip + k])
                ib += 1
                ip += k
        return EcpSystem(self.geometry.copy(), sE, K, lE, nE, dE, aE, sB, lB, KB, dB, aB,
                         self.largeGridOrder, self.tolerance, self.accuracy,
                         name=self.name + "[subset]")


# ---------------------------------------------------------------- builders

class _Builder:
    def __init__(self):
        self.geom, self.sE, self.K, self.lE, self.nE, self.dE, self.aE = [], [], [], [], [], [], []
        self.sB, self.lB, self.KB, self.dB, self.aB = [], [], [], [], []

    def atom(self, xyz, ecp=None, shells=None):
        """ecp: list of (l, [(n, d, a), ...]); shells: list of (l, [(d, a), ...])."""
        self.geom.append(np.asarray(xyz, dtype=np.float64))
        ecp = ecp or []
        shells = shells or []
        self.sE.append(len(ecp))
        for l, terms in ecp:
            self.K.append(len(terms)); self.lE.append(l)
            for n, d, a in terms:
                self.nE.append(n); self.dE.append(d); self.aE.append(a)
        self.sB.append(len(shells))
        for l, prims in shells:
            self.lB.append(l); self.KB.append(len(prims))
            for d, a in prims:
                self.dB.append(d); self.aB.append(a)

    def build(self, name, **kw) -> EcpSystem:
        return EcpSystem(np.concatenate(self.geom), self.sE, self.K, self.lE, self.nE, self.dE,
                         self.aE, self.sB, self.lB, self.KB, self.dB, self.aB, name=name, **kw)


def _loguniform(rng, lo, hi, size=None):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size))


def _ecp_channels(rng, L, nterms, zlo=0.1, zhi=20.0):
    """Channels l = 0..L (l = L is the local part); per term: n, z, d in that order."""
    out = []
    for l in range(L + 1):
        k = nterms if isinstance(nterms, int) else int(rng.integers(nterms[0], nterms[1] + 1))
        terms = []
        for _ in range(k):
            n = float(rng.integers(0, 3))
            z = float(_loguniform(rng, zlo, zhi))
            d = float(rng.uniform(-10.0, 10.0))
            terms.append((n, d, z))
        out.append((l, terms))
    return out


def _shell(rng, l, nprim, elo, ehi):
    """One contracted shell: exponents then coefficients, per primitive in order."""
    prims = []
    for _ in range(nprim):
        a = float(_loguniform(rng, elo, ehi))
        d = float(rng.uniform(0.1, 1.0))
        prims.append((d, a))
    return (l, prims)


def example_like(seed: int = 0) -> EcpSystem:
    """Single-centre system shaped like the reference's example.

    One ECP centre at the origin without basis functions; channels l = 0..3
    semi-local plus the local channel l = 4, three terms each (n in {0,1,2},
    exponent log-uniform [0.1, 20], coefficient uniform [-10, 10]); four atoms
    uniform in the cube [-2, 2]^3 bohr, each with s, p and d shells of three
    primitives (exponents log-uniform [0.05, 50], coefficients uniform
    [0.1, 1]).  12 shells, 78 shell pairs, one centre.
    """
    rng = np.random.default_rng(seed)
    b = _Builder()
    b.atom([0.0, 0.0, 0.0], ecp=_ecp_channels(rng, 4, 3))
    for _ in range(4):
        xyz = rng.uniform(-2.0, 2.0, 3)
        b.atom(xyz, shells=[_shell(rng, l, 3, 0.05, 50.0) for l in (0, 1, 2)])
    return b.build(f"example_like(seed={seed})")


def batched_cluster(seed: int = 0, n_centres: int = 50, n_basis_atoms: int = 21,
                    shells_per_atom: int = 3, box: float = 12.0, lmax_ecp: int = 4,
                    l_weights=(0.4, 0.3, 0.2, 0.1), kmax: int = 8) -> EcpSystem:
    """Batched FP64 workload: 50 ECP centres in a random cluster.

    Atoms are placed uniformly in a cube of side `box` bohr (about 20 atoms
    within 6 bohr of each centre).  Every atom carries an ECP with L drawn
    uniformly from 1..lmax_ecp (the first has L = lmax_ecp), 2-6 terms per
    channel.  The first `n_basis_atoms` atoms also carry `shells_per_atom`
    contracted shells with l drawn with weights 0.4/0.3/0.2/0.1 and contraction
    length uniform 1..kmax: 63 shells give 2016 shell pairs.
    """
    rng = np.random.default_rng(seed)
    b = _Builder()
    n_atoms = max(n_centres, n_basis_atoms)
    for i in range(n_atoms):
        xyz = rng.uniform(-box / 2, box / 2, 3)
        ecp = None
        if i < n_centres:
            L = lmax_ecp if i == 0 else int(rng.integers(1, lmax_ecp + 1))
            ecp = _ecp_channels(rng, L, (2, 6))
        shells = None
        if i < n_basis_atoms:
            shells = []
            for _ in range(shells_per_atom):
                l = int(rng.choice(len(l_weights), p=np.asarray(l_weights) / sum(l_weights)))
                k = int(rng.integers(1, kmax + 1))
                shells.append(_shell(rng, l, k, 0.05, 50.0))
        b.atom(xyz, ecp=ecp, shells=shells)
    return b.build(f"batched_cluster(seed={seed})")


def random_system(seed: int, n_atoms: int = 4, n_centres: int = 2, lmax_basis: int = 2,
                  lmax_ecp: int = 3, kmax: int = 3, box: float = 5.0, elo=0.05, ehi=50.0,
                  ecp_on_basis_atom: bool = True, nterms=(1, 3)) -> EcpSystem:
    """Small mixed system for parity tests (ECP centres may carry basis shells)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    for i in range(n_atoms):
        xyz = rng.uniform(-box / 2, box / 2, 3)
        ecp = None
        if i < n_centres:
            L = lmax_ecp if i == 0 else int(rng.integers(1, lmax_ecp + 1))
            ecp = _ecp_channels(rng, L, nterms)
        shells = None
        if ecp_on_basis_atom or i >= n_centres:
            nsh = int(rng.integers(1, 4))
            shells = [_shell(rng, int(rng.integers(0, lmax_basis + 1)),
                             int(rng.integers(1, kmax + 1)), elo, ehi) for _ in range(nsh)]
        b.atom(xyz, ecp=ecp, shells=shells)
    return b.build(f"random_system(seed={seed})")


def mixed_batch(seed: int = 0, n_shells: int = 200, n_centres: int = 10, box: float = 14.0,
                lmax_basis: int = 4, kmax: int = 10, lmax_ecp: int = 4) -> EcpSystem:
    """Large mixed-precision batch: l up to 4, contraction 1..10, exponents
    log-uniform [0.02, 200]; 200 shells on 50 atoms give 20100 shell pairs."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    n_atoms = max(n_centres, (n_shells + 3) // 4)
    per_atom = [n_shells // n_atoms + (1 if i < n_shells % n_atoms else 0) for i in range(n_atoms)]
    for i in range(n_atoms):
        xyz = rng.uniform(-box / 2, box / 2, 3)
        ecp = None
        if i < n_centres:
            L = lmax_ecp if i == 0 else int(rng.integers(1, lmax_ecp + 1))
            ecp = _ecp_channels(rng, L, (2, 6))
        shells = [_shell(rng, int(rng.integers(0, lmax_basis + 1)), int(rng.integers(1, kmax + 1)),
                         0.02, 200.0) for _ in range(per_atom[i])]
        b.atom(xyz, ecp=ecp, shells=shells)
    return b.build(f"mixed_batch(seed={seed})")


def large_sweep(seed: int = 0, n_shells: int = 447, n_centres: int = 4, box: float = 16.0,
                kmax: int = 6) -> EcpSystem:
    """High-accuracy sweep: 447 shells (about 100,000 shell pairs) with l up to 4,
    ECP channels up to L = 5 with 6 terms each, exponents log-uniform
    [0.01, 500], quadrature tolerance 1e-12."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    n_atoms = max(n_centres, (n_shells + 4) // 5)
    per_atom = [n_shells // n_atoms + (1 if i < n_shells % n_atoms else 0) for i in range(n_atoms)]
    for i in range(n_atoms):
        xyz = rng.uniform(-box / 2, box / 2, 3)
        ecp = None
        if i < n_centres:
            L = 5 if i == 0 else int(rng.integers(1, 6))
            ecp = _ecp_channels(rng, L, 6)
        shells = [_shell(rng, int(rng.integers(0, 5)), int(rng.integers(1, kmax + 1)), 0.01, 500.0)
                  for _ in range(per_atom[i])]
        b.atom(xyz, ecp=ecp, shells=shells)
    return b.build(f"large_sweep(seed={seed})")


def serving_molecule(rng: np.random.Generator, n_atoms: int, n_centres: int) -> EcpSystem:
    """One request of the serving stream: s..f basis with 1..6 primitives,
    1..n_centres ECP centres (L up to 4, 2-6 terms), atoms about 2.5 bohr apart."""
    b = _Builder()
    box = 2.5 * n_atoms ** (1.0 / 3.0) + 2.0
    for i in range(n_atoms):
        xyz = rng.uniform(-box / 2, box / 2, 3)
        ecp = _ecp_channels(rng, int(rng.integers(1, 5)), (2, 6)) if i < n_centres else None
        nsh = int(rng.integers(1, 4))
        shells = [_shell(rng, int(rng.integers(0, 4)), int(rng.integers(1, 7)), 0.05, 50.0)
                  for _ in range(nsh)]
        b.atom(xyz, ecp=ecp, shells=shells)
    return b.build(f"serving(n_atoms={n_atoms})")

"""Parity of the CUDA path (through the C ABI) with the reference fixtures and
the oracle.  Bar: max abs error <= 1e-10 per block element (FP64 path)."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import TOL_ABS, golden_files, load_golden, one_centre_answers, one_centre_system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()  # raises if the CUDA library is missing: no silent fallback
    return libecp_gb300


def assert_blocks_match(meta, data, meta_ref, data_ref, tol=TOL_ABS):
    assert meta.shape == meta_ref.shape, (meta.shape, meta_ref.shape)
    assert np.array_equal(meta, meta_ref)
    err = np.max(np.abs(data - data_ref)) if data.size else 0.0
    assert err <= tol, err


@pytest.mark.parametrize("name", golden_files())
def test_blocks_match_reference_fixtures(eg, name):
    s, z = load_golden(name)
    meta, data = eg.blocks(s)
    assert_blocks_match(meta, data, z["meta"], z["data"])
    if "matrix" in z:
        I = eg.get_integrals(s)
        assert np.max(np.abs(I - z["matrix"])) <= TOL_ABS


CASES = [
    dict(seed=10, n_atoms=4, n_centres=2, lmax_basis=2, lmax_ecp=3),
    dict(seed=11, n_atoms=5, n_centres=3, lmax_basis=1, lmax_ecp=2),
    dict(seed=12, n_atoms=3, n_centres=1, lmax_basis=3, lmax_ecp=4, kmax=4),
    dict(seed=13, n_atoms=3, n_centres=3, lmax_basis=2, lmax_ecp=1, kmax=5),
    dict(seed=14, n_atoms=2, n_centres=2, lmax_basis=4, lmax_ecp=5, kmax=3),
    dict(seed=15, n_atoms=3, n_centres=2, lmax_basis=4, lmax_ecp=2, kmax=2),   # l >= L
    dict(seed=16, n_atoms=4, n_centres=2, lmax_basis=3, lmax_ecp=4, elo=0.01, ehi=500),
    dict(seed=17, n_atoms=4, n_centres=2, lmax_basis=2, lmax_ecp=3, box=12.0),  # sparse
    dict(seed=18, n_atoms=4, n_centres=4, lmax_basis=2, lmax_ecp=3, box=1.5),   # dense
    dict(seed=19, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3, ecp_on_basis_atom=False),
]


@pytest.mark.parametrize("kw", CASES, ids=[f"seed{c['seed']}" for c in CASES])
def test_blocks_match_oracle(eg, kw):
    kw = dict(kw)
    s = W.random_system(kw.pop("seed"), **kw)
    rc, mo, do = O.oracle_blocks(s)
    assert rc == 0
    meta, data = eg.blocks(s)
    assert_blocks_match(meta, data, mo, do)


def test_one_centre_known_answers(eg):
    s, _, _ = one_centre_system()
    I = eg.get_integrals(s)
    for (i, j), v in one_centre_answers().items():
        assert abs(I[i, j] - v) <= 1e-12 * max(1.0, abs(v)), (i, j, I[i, j], v)


def test_getintegrals_accumulates_upper_triangle(eg):
    """I += blocks where row <= col; lower triangle and padding untouched;
    rowdim may exceed the basis dimension."""
    s = W.random_system(21, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    n, rowdim = s.dim, s.dim + 5
    rc, ref = O.oracle_matrix(s)
    rng = np.random.default_rng(0)
    I0 = rng.normal(size=(n + 2, rowdim))
    I = I0.copy()
    assert eg.lib().getIntegrals(*eg._ptrs(s), rowdim, I.ctypes.data_as(eg._D)) == 0
    delta = I - I0
    assert np.max(np.abs(delta[:n, :n] - ref)) <= TOL_ABS
    assert np.all(delta[:, n:] == 0) and np.all(delta[n:, :] == 0)
    assert np.all(np.tril(delta[:n, :n], -1) == 0)


def test_callback_interface_order_and_values(eg):
    s = W.random_system(22, n_atoms=4, n_centres=2, lmax_basis=2, lmax_ecp=3)
    rc, meta, data = eg.calculate_blocks_via_callback(s)
    assert rc == 0
    rco, mo, do = O.oracle_blocks(s)
    assert_blocks_match(meta, data, mo, do)


def test_local_only_centre(eg):
    """A centre with only a local channel (L = 0): the reference aborts on it
    (zero-sized table); the engine computes the type-1 part and a zero type-2
    block, like the oracle."""
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=[(0, [(2.0, 2.0, 1.1)])], shells=[(1, [(0.7, 0.9)])])
    b.atom([0.5, -0.3, 0.8], shells=[(0, [(0.5, 0.4), (0.3, 2.0)]), (2, [(1.0, 0.6)])])
    s = b.build("local_only")
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s)
    assert_blocks_match(meta, data, mo, do)


def test_parameters_other_than_defaults(eg):
    """largeGridOrder 2048, looser tolerance, other accuracy, non-integer r^n."""
    s = W.random_system(23, n_atoms=3, n_centres=2, lmax_basis=2, lmax_ecp=3)
    s.nECP[::3] += 0.5
    s.largeGridOrder, s.tolerance, s.accuracy = 2048, 1e-10, 1e-12
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s)
    assert_blocks_match(meta, data, mo, do)


def test_maximum_sizes(eg):
    """g shells with contraction 16 against a 5-channel ECP (largest class)."""
    rng = np.random.default_rng(5)
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=W._ecp_channels(rng, 5, 2),
           shells=[W._shell(rng, 4, 16, 0.05, 50.0)])
    b.atom([1.1, 0.4, -0.6], shells=[W._shell(rng, 4, 3, 0.05, 50.0), W._shell(rng, 0, 2, 0.1, 5)])
    s = b.build("max")
    rc, mo, do = O.oracle_blocks(s)
    meta, data = eg.blocks(s)
    assert_blocks_match(meta, data, mo, do)


def test_sizes_beyond_limits_are_rejected(eg):
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=[(0, [(2.0, 1.0, 1.0)])], shells=[(5, [(1.0, 1.0)])])
    with pytest.raises(RuntimeError, match="basis l=5"):
        eg.blocks(b.build("h shell"))


def test_empty_inputs(eg):
    """No ECP centre, or no basis functions: nothing is added."""
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], shells=[(0, [(1.0, 1.0)])])
    s = b.build("no ecp")
    I = np.full((s.dim, s.dim), 3.0)
    eg.get_integrals(s, I)
    assert np.all(I == 3.0)
    meta, data = eg.blocks(s)
    assert meta.shape == (0, 8)


def test_deterministic(eg):
    s = W.random_system(24, n_atoms=4, n_centres=3, lmax_basis=3, lmax_ecp=3)
    _, d1 = eg.blocks(s)
    _, d2 = eg.blocks(s)
    assert np.array_equal(d1, d2)


def test_full_cluster_sampled_units(eg):
    """Full 50-centre, 2016-pair workload on the GPU; a seeded sample of
    units checked against the oracle run on the unit's own sub-system (the
    centre and the two atoms), which gives the same block as the full system."""
    s = W.batched_cluster(0)
    meta, data, status, info = eg.blocks(s, with_status=True)
    assert (status != eg.UNIT_SKIPPED).sum() * 2 == len(meta)
    offs = np.concatenate([[0], np.cumsum([(m[2] + 1) * (m[2] + 2) // 2 * (m[5] + 1) * (m[5] + 2) // 2
                                           for m in meta])])
    index = {tuple(m[[6, 0, 1, 3, 4, 7]]): i for i, m in enumerate(meta)}
    rng = np.random.default_rng(1)
    picks = rng.choice(len(meta) // 2, size=16, replace=False) * 2
    for i in picks:
        A, s1, la, B, s2, lb, C, _ = meta[i]
        sub = s.subset(centres=[C], basis_atoms=[A, B])
        rc, mo, do = O.oracle_blocks(sub)
        assert rc == 0
        for j, m in enumerate(O.split_blocks(mo, do)):
            key, blk = m
            if key[1:5] == (A, s1, B, s2):
                k = index[key]
                got = data[offs[k]:offs[k + 1]].reshape(blk.shape)
                assert np.max(np.abs(got - blk)) <= TOL_ABS


def test_job_rerun_matches_one_call(eg):
    s = W.random_system(25, n_atoms=4, n_centres=2, lmax_basis=2, lmax_ecp=3)
    job = eg.Job(s)
    ms, mu = job.run(2, flush_l2=True)
    assert np.all(ms > 0) and np.all(mu > 0) and np.all(mu <= ms)
    I = job.matrix()
    job.close()
    assert np.array_equal(I, eg.get_integrals(s))


def test_forced_non_convergence_is_reported(eg):
    """A tolerance no quadrature can meet makes every large-grid quadrature run
    out of levels.  The reference then reads a freed table and aborts; the
    engine keeps each quadrature's full-grid estimate (as the oracle does),
    flags the units, and still hands out every block.  getIntegrals keeps the
    reference's contract (returns 0), ecpgb_getIntegrals returns 2 and the
    handle interface returns the reference's type-1 error code 1."""
    s = W.random_system(26, n_atoms=2, n_centres=1, lmax_basis=1, lmax_ecp=2)
    s.tolerance = 1e-300
    meta, data, status, info = eg.blocks(s, with_status=True)
    assert info["firstFailed"] >= 0
    assert eg.UNIT_WARN_TYPE1 in set(np.unique(status))
    rc, mo, do, st = O.oracle_blocks(s, with_stats=True)
    assert st["psm92_failed"] > 0
    assert_blocks_match(meta, data, mo, do)
    rc, I, info2 = eg.get_integrals_info(s)
    assert rc == 2
    rc, meta_cb, data_cb = eg.calculate_blocks_via_callback(s)
    assert rc == 1 and np.array_equal(meta_cb, mo)
    I = np.zeros((s.dim, s.dim))
    assert eg.lib().getIntegrals(*eg._ptrs(s), s.dim, I.ctypes.data_as(eg._D)) == 0


def test_unit_where_the_reference_aborts(eg):
    """Centre 0 with atoms 1 and 6 of the batched cluster: a type-2 large-grid
    quadrature exhausts its levels and the reference aborts (heap corruption
    after its use of a freed table).  Engine and oracle agree on the
    full-grid estimate."""
    s = W.batched_cluster(0).subset(centres=[0], basis_atoms=[1, 6])
    rc, mo, do, st = O.oracle_blocks(s, with_stats=True)
    assert st["psm92_failed"] >= 1
    meta, data, status, info = eg.blocks(s, with_status=True)
    assert info["firstFailed"] >= 0
    assert_blocks_match(meta, data, mo, do)

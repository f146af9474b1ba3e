"""Readers of the example program's text inputs (xyz, ECP, basis; no GPU):
both ECP term layouts, round trip of a seeded system, and errors for missing
files and malformed lines."""
import numpy as np
import pytest

from libecp_gb300 import workloads as W


@pytest.fixture(scope="module")
def eg():
    import libecp_gb300
    libecp_gb300.lib()
    return libecp_gb300


def write_inputs(tmp_path, s, ecp_layout=4, blank_comment=False):
    xyz = tmp_path / "s.xyz"
    lines = [str(s.n_atoms), "" if blank_comment else "seeded system"]
    g = s.geometry.reshape(-1, 3)
    for a in range(s.n_atoms):
        lines.append(f"X{a} {float(g[a, 0])!r} {float(g[a, 1])!r} {float(g[a, 2])!r}")
    xyz.write_text("\n".join(lines) + "\n")
    ecp, t, sh = [], 0, 0
    for a in range(s.n_atoms):
        ns = int(s.shellsECP[a])
        ecp.append(f"{a + 1} 2 {ns}")
        for _ in range(ns):
            l, k = int(s.lECP[sh]), int(s.KECP[sh])
            ecp.append(f"  {l} {k}\t\t   ")
            for i in range(k):
                a_, d_, n_ = float(s.aECP[t]), float(s.dECP[t]), float(s.nECP[t])
                ecp.append(f"  {i + 1} {a_!r} {d_!r} {n_!r}" if ecp_layout == 4 else f"   {d_!r}   {a_!r}  {n_!r}")
                t += 1
            sh += 1
    (tmp_path / "s.ecp").write_text("\n".join(ecp) + "\n")
    bs, p, sh = [], 0, 0
    for a in range(s.n_atoms):
        ns = int(s.shellsBS[a])
        bs.append(f"{a + 1} {ns}")
        for _ in range(ns):
            l, k = int(s.lBS[sh]), int(s.KBS[sh])
            bs.append(f" {l} {k}")
            for i in range(k):
                bs.append(f"  {i + 1}  {float(s.aBS[p])!r}  {float(s.dBS[p])!r}")
                p += 1
            sh += 1
    (tmp_path / "s.bs").write_text("\n".join(bs) + "\n")
    return str(xyz), str(tmp_path / "s.ecp"), str(tmp_path / "s.bs")


@pytest.mark.parametrize("layout", [4, 3])
@pytest.mark.parametrize("blank", [False, True])
def test_round_trip(eg, tmp_path, layout, blank):
    s = W.random_system(7, n_atoms=4, n_centres=2, lmax_basis=3, lmax_ecp=3)
    got, symbols = eg.load_system(*write_inputs(tmp_path, s, layout, blank))
    assert symbols == [f"X{a}" for a in range(s.n_atoms)]
    for k in ("geometry", "shellsECP", "KECP", "lECP", "nECP", "dECP", "aECP", "shellsBS", "lBS", "KBS",
              "dBS", "aBS"):
        assert np.array_equal(getattr(got, k), getattr(s, k)), k
    assert (got.largeGridOrder, got.tolerance, got.accuracy) == (1024, 1e-12, 1e-14)


def test_three_number_terms_are_coefficient_exponent_power(eg, tmp_path):
    (tmp_path / "c.xyz").write_text("1\ncarbon\nC 0.0 0.0 0.0\n")
    (tmp_path / "c.ecp").write_text("6 2 2\n  0 1 \n   37.4565   6.8446  2\n  1 1\n  1  7.9  -2.67  2\n")
    (tmp_path / "c.bs").write_text("6 1\n 0 1\n  1  0.5  1.0\n")
    s, _ = eg.load_system(str(tmp_path / "c.xyz"), str(tmp_path / "c.ecp"), str(tmp_path / "c.bs"))
    assert list(s.dECP) == [37.4565, -2.67] and list(s.aECP) == [6.8446, 7.9] and list(s.nECP) == [2, 2]


def test_errors(eg, tmp_path):
    s = W.random_system(8, n_atoms=2, n_centres=1, lmax_basis=1, lmax_ecp=2)
    xyz, ecp, bs = write_inputs(tmp_path, s)
    with pytest.raises(RuntimeError, match="cannot open"):
        eg.load_system(str(tmp_path / "missing.xyz"), ecp, bs)
    (tmp_path / "bad.bs").write_text("1 1\n 0 2\n  1 0.5 1.0\n")  # truncated, and atom 2 missing
    with pytest.raises(RuntimeError, match="end of file"):
        eg.load_system(xyz, ecp, str(tmp_path / "bad.bs"))
    (tmp_path / "bad.ecp").write_text("1 2 1\n 0 1\n  0.5 1.0\n")
    with pytest.raises(RuntimeError, match="fields"):
        eg.load_system(xyz, str(tmp_path / "bad.ecp"), bs)
    (tmp_path / "bad.xyz").write_text("3\ncomment\nC 0 0 0\n")
    with pytest.raises(RuntimeError, match="atoms announced"):
        eg.load_system(str(tmp_path / "bad.xyz"), ecp, bs)

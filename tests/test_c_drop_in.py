"""The drop-in from C: a host program compiled against include/ and linked
to libecp_gb300.so as it would link the reference's libecp.a.  On the CPU it
must compile and link; on a GPU its getIntegrals matrix and callback blocks
must equal those of the Python binding."""
import os
import subprocess

import numpy as np
import pytest

from libecp_gb300 import workloads as W
from tests.helpers import ROOT

SRC = os.path.join(ROOT, "tests", "c", "drop_in.c")
LIBDIR = os.path.join(ROOT, "libecp_gb300")


def build(tmp_path):
    exe = str(tmp_path / "drop_in")
    cmd = ["gcc", "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-lecp_gb300", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compiles_and_links(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libecp_gb300.so")):
        subprocess.run(["python", "-m", "libecp_gb300.build"], cwd=ROOT, check=True)
    build(tmp_path)  # libecp_gb300.so: -lecp_gb300 finds it


def the_system():
    b = W._Builder()
    b.atom([0.0, 0.0, 0.0], ecp=[(0, [(2.0, 3.0, 1.3), (1.0, -1.2, 0.4)]), (1, [(2.0, -2.0, 0.7)]),
                                 (2, [(2.0, 1.5, 2.1), (0.0, 0.4, 0.9)])])
    b.atom([0.9, -0.4, 0.3], shells=[(0, [(0.6, 1.7), (0.4, 0.3)]), (1, [(0.9, 0.8)])])
    b.atom([-0.7, 0.5, 0.8], shells=[(0, [(0.7, 1.1)]), (1, [(0.5, 2.4), (0.8, 0.6)])])
    return b.build("drop_in")


@pytest.mark.gpu
def test_matches_python_binding(tmp_path):
    import libecp_gb300 as eg
    exe = build(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    s = the_system()
    I = eg.get_integrals(s)
    rcm, meta, data = eg.calculate_blocks_via_callback(s)
    assert "RC 0" in out and "CB 0" in out
    Ic = np.zeros_like(I)
    for line in out:
        f = line.split()
        if f[0] == "M":
            Ic[int(f[1]), int(f[2])] = float(f[3])
    assert np.array_equal(Ic, np.triu(I))
    firsts, off = [], 0
    for m in meta:
        firsts.append(data[off])
        off += (m[2] + 1) * (m[2] + 2) // 2 * ((m[5] + 1) * (m[5] + 2) // 2)
    cb = [float(l.split()[-1]) for l in out if l.startswith("B ")]
    assert np.array_equal(np.array(cb), np.array(firsts))


@pytest.mark.gpu
def test_environment_selects_the_batched_engine(tmp_path):
    """LIBECP_GB300_MODE=fast: the unchanged host program runs on the batched
    engine; its matrix and callback blocks agree with the default run within
    the FP64 bar."""
    exe = build(tmp_path)

    def run(mode):
        env = dict(os.environ)
        if mode is None:
            env.pop("LIBECP_GB300_MODE", None)
        else:
            env["LIBECP_GB300_MODE"] = mode
        out = subprocess.run([exe], capture_output=True, text=True, check=True, env=env)
        return out.stdout.splitlines(), out.stderr

    base, _ = run(None)
    fast, _ = run("fast")
    assert "RC 0" in fast and "CB 0" in fast
    vals = lambda out: np.array([float(l.split()[-1]) for l in out if l.startswith(("M ", "B "))])
    assert len(vals(base)) == len(vals(fast)) > 0
    assert np.max(np.abs(vals(base) - vals(fast))) <= 1e-10
    bad, err = run("bogus")
    assert "not fp64, fast or mixed" in err and "RC 0" in bad

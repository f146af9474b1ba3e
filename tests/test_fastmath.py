"""fast_exp (libecp_gb300/csrc/ecp_fastmath.h) against the C library's exp.

The header is compiled for the host here; every operation in it (fma, add,
integer and bit manipulation) is IEEE-defined, so the device build computes
the same values."""
import os
import subprocess

import pytest

from tests.helpers import ROOT

SRC = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "ecp_fastmath.h"
static int64_t ord(double x) { int64_t i; std::memcpy(&i, &x, 8); return i < 0 ? INT64_MIN - i : i; }
int main() {
  double worst = 0, at = 0; long n = 0;
  uint64_t s = 88172645463325252ull;
  for (long k = 0; k < 4000000; k++) {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    double u = (double)(s >> 11) / 9007199254740992.0;
    double x = k % 4 == 0 ? -745.0 + 1454.0 * u : (k % 4 == 1 ? -40.0 + 45.0 * u : -1.0 + 2.0 * u);
    double a = ecpgb::fast_exp(x), b = std::exp(x);
    if (b < 2.3e-308) continue;  // subnormal range: absolute error checked below
    double ulp = std::fabs((double)(ord(a) - ord(b)));
    if (ulp > worst) { worst = ulp; at = x; }
    n++;
  }
  double sub = 0;
  for (double x = -745.0; x < -708.0; x += 0.001) sub = std::fmax(sub, std::fabs(ecpgb::fast_exp(x) - std::exp(x)));
  // the overflow threshold: finite (within 2 ulp) up to ln(DBL_MAX), infinite above
  int over = 0;
  for (double x = 709.7; x < 709.79; x += 1e-5) {
    double a = ecpgb::fast_exp(x), b = std::exp(x);
    if (std::isinf(a) != std::isinf(b) || (!std::isinf(b) && std::fabs((double)(ord(a) - ord(b))) > 2.0)) over++;
  }
  const double lnmax = 0x1.62e42fefa39efp+9;
  over += std::isinf(ecpgb::fast_exp(lnmax)) + !std::isinf(ecpgb::fast_exp(std::nextafter(lnmax, 800.0)));
  std::printf("%ld %.1f %.17g %.3g %.17g %.17g %d\n", n, worst, at, sub, ecpgb::fast_exp(0.0), ecpgb::fast_exp(-1e-20), over);
  return 0;
}
"""


def test_fast_exp_against_libm(tmp_path):
    src, exe = str(tmp_path / "t.cpp"), str(tmp_path / "t")
    with open(src, "w") as f:
        f.write(SRC)
    inc = os.path.join(ROOT, "libecp_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe],
                       capture_output=True, text=True)
    if r.returncode:
        pytest.fail(r.stderr)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    n, worst, sub = int(out[0]), float(out[1]), float(out[3])
    assert n > 3_000_000
    assert worst <= 2.0, f"max error {worst} ulp at x = {out[2]}"
    assert sub < 1e-320
    assert float(out[4]) == 1.0 and float(out[5]) == 1.0
    assert int(out[6]) == 0, "overflow threshold differs from exp's"

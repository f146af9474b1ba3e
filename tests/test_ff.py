"""Double-single arithmetic of the mixed-precision path
(libecp_gb300/csrc/ecp_ff.h), compiled for the host: the error-free
transformations are exact, the compound operations and the exp stay within
their stated relative errors against FP64.

Every operation in the header is an IEEE float add, multiply or FMA (no
contraction: -ffp-contract=off here, explicit __fadd_rn/__fmul_rn on the
device), so the device computes the same values."""
import os
import subprocess

import pytest

from tests.helpers import ROOT

SRC = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include "ecp_ff.h"
using namespace ecpgb;
static uint64_t s = 0x9E3779B97F4A7C15ull;
static double uni() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return (double)(s >> 11) / 9007199254740992.0; }
static float rf(double lo, double hi) { return (float)(lo + (hi - lo) * uni()); }
static ff rff(double lo, double hi) { return ff_from_double(lo + (hi - lo) * uni()); }
static double rel(double a, double b) { return b == 0.0 ? std::fabs(a) : std::fabs(a - b) / std::fabs(b); }
int main() {
  long inexact = 0;
  double e_add = 0, e_mul = 0, e_mulf = 0, e_exp = 0, e_sum = 0, e_split = 0, e_low = 0;
  for (int k = 0; k < 1000000; k++) {
    const float a = rf(-1e3, 1e3), b = rf(-1e3, 1e3) * (float)std::ldexp(1.0, (int)(uni() * 40) - 20);
    // two-sum and two-prod are exact: hi + lo equals the exact result
    ff t = two_sum(a, b), p = two_prod(a, b);
    if ((double)t.hi + (double)t.lo != (double)a + (double)b) inexact++;
    if ((double)p.hi + (double)p.lo != (double)a * (double)b) inexact++;
    if (std::fabs(a) >= std::fabs(b)) {
      ff f = fast_two_sum(a, b);
      if ((double)f.hi + (double)f.lo != (double)a + (double)b) inexact++;
    }
    // compound operations against FP64 on the ff inputs' exact values
    const ff x = rff(0.5, 4.0), y = rff(0.5, 4.0);
    const double xd = ff_to_double(x), yd = ff_to_double(y);
    e_add = std::fmax(e_add, rel(ff_to_double(ff_add(x, y)), xd + yd));
    e_mul = std::fmax(e_mul, rel(ff_to_double(ff_mul(x, y)), xd * yd));
    e_mulf = std::fmax(e_mulf, rel(ff_to_double(ff_mul_f(x, a)), xd * (double)a));
    // exp: relative error where the result's low float is a normal float
    // (results above 2^-100, x > -69); below that, down to the cut at -87,
    // the low part leaves the float range and the absolute error is what
    // bounds the contribution
    const double d = -69.0 * uni() + (k % 8 == 0 ? 1.0 * uni() : 0.0);
    const ff dx = ff_from_double(d);
    e_exp = std::fmax(e_exp, rel(ff_to_double(ff_exp(dx)), std::exp(ff_to_double(dx))));
    const ff dl = ff_from_double(-69.0 - 18.0 * uni());
    e_low = std::fmax(e_low, std::fabs(ff_to_double(ff_exp(dl)) - std::exp(ff_to_double(dl))));
    e_split = std::fmax(e_split, rel(ff_to_double(ff_from_double(d)), d));
  }
  // the compensated sum of 10,000 terms of mixed sign
  for (int r = 0; r < 200; r++) {
    ff_acc acc;
    double ref = 0.0, mag = 0.0;
    for (int i = 0; i < 10000; i++) {
      const ff v = rff(-1.0, 1.0);
      acc.add(v);
      ref += ff_to_double(v);
      mag += std::fabs(ff_to_double(v));
    }
    e_sum = std::fmax(e_sum, std::fabs(acc.value() - ref) / mag);
  }
  std::printf("%ld %.3g %.3g %.3g %.3g %.3g %.3g %.3g\n", inexact, e_add, e_mul, e_mulf, e_exp, e_sum, e_split, e_low);
  return 0;
}
"""


def test_double_single_arithmetic(tmp_path):
    src, exe = str(tmp_path / "t.cpp"), str(tmp_path / "t")
    with open(src, "w") as f:
        f.write(SRC)
    inc = os.path.join(ROOT, "libecp_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe],
                       capture_output=True, text=True)
    if r.returncode:
        pytest.fail(r.stderr)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    inexact = int(out[0])
    e_add, e_mul, e_mulf, e_exp, e_sum, e_split, e_low = (float(v) for v in out[1:])
    assert inexact == 0, "an error-free transformation lost bits"
    assert e_split <= 2.0 ** -47, e_split          # a double split into two floats
    assert e_add <= 2.0 ** -45 and e_mul <= 2.0 ** -45 and e_mulf <= 2.0 ** -45, (e_add, e_mul, e_mulf)
    assert e_exp <= 2.0 ** -44, e_exp               # Tang's method in double-single
    assert e_low <= 2.0 ** -140, e_low              # results below 2^-100: absolute error
    # Sum2 over 10,000 terms: within n 2^-48 of the sum of magnitudes (its
    # error bound), far below plain FP32 summation's n 2^-24
    assert e_sum <= 1e4 * 2.0 ** -48, e_sum

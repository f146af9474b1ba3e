// ecp_fastmath.h -- FP64 exp for the batched path (host and device).
//
// Table-driven method of P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15 (1989)
// 144-157, written here from that description, with a 512-entry table:
//   x = (512 m + j) ln2/512 + r,  |r| <= ln2/1024,
//   exp(x) = 2^m * 2^(j/512) * exp(r),
// with exp(r) - 1 from its degree-4 Taylor polynomial (truncation below
// 1.3e-18 relative on |r| <= ln2/1024), the table rounded to nearest and the
// reduction done with a two-part ln2/512 whose leading part has 32
// significant bits, so n * L1 is exact (ecp_exp2_table.h, written by
// gen_exp2_table.py).  The integer n comes out of one FMA against 1.5 * 2^52
// (round to nearest of the exact product), the range test is an integer test
// on the high word, and 2^m enters through the exponent field of the table
// value, so the common case takes 9 FP64 operations -- on GB300 FP64 runs at
// 1/64 of the FP32 rate and every one counts.  Maximum error about 1.5 ulp;
// tests/test_fastmath.py measures it against the C library's exp.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "ecp_exp2_table.h"

#ifdef __CUDACC__
#define ECPGB_HD __host__ __device__ __forceinline__
#else
#define ECPGB_HD inline
#endif

namespace ecpgb {

#ifdef __CUDACC__
static __device__ const double kExp2TableDev[ECPGB_EXP2_N] = ECPGB_EXP2_TABLE;
#endif
static const double kExp2TableHost[ECPGB_EXP2_N] = ECPGB_EXP2_TABLE;

ECPGB_HD long long dbits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

ECPGB_HD double bits_d(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

ECPGB_HD double pow2i(int m) { return bits_d((long long)(m + 1023) << 52); }  // -1022 <= m <= 1023

ECPGB_HD double fast_exp(double x) {
  const double shifter = 0x1.8p52;
  // |x| < 708 (and not NaN): the result and 2^m are normal
  const bool common = (int)((unsigned long long)dbits(x) >> 32 & 0x7fffffffu) < 0x40862000;
  if (__builtin_expect(!common, 0)) {  // rare: |x| >= 708, NaN
    if (!(x > -745.2)) return (x != x) ? x : 0.0;  // NaN stays NaN, underflow to 0
    // overflow exactly where exp overflows: above ln(DBL_MAX) rounded to
    // the nearest double (a result of 0 * exp(x) is 0 below it, NaN above)
    if (x > 0x1.62e42fefa39efp+9) return HUGE_VAL;
  }
  const double t = std::fma(x, ECPGB_EXP2_INV, shifter);
  const int n = (int)dbits(t);  // low word of t: the nearest integer to x * 512 / ln2
  const double tn = t - shifter;
  double r = std::fma(-tn, ECPGB_EXP2_L1, x);
  r = std::fma(-tn, ECPGB_EXP2_L2, r);
  const int j = n & (ECPGB_EXP2_N - 1), m = n >> ECPGB_EXP2_LOG2N;
  double p = std::fma(r, 1.0 / 24.0, 1.0 / 6.0);
  p = std::fma(p, r, 0.5);
  p = std::fma(p, r, 1.0);
  p = p * r;  // exp(r) - 1
#ifdef __CUDA_ARCH__
  const double s = kExp2TableDev[j];
#else
  const double s = kExp2TableHost[j];
#endif
  if (common) {
    const double sm = bits_d(dbits(s) + ((long long)m << 52));  // s * 2^m, exact
    return std::fma(sm, p, sm);
  }
  const double y = std::fma(s, p, s);
  if (m > 1023) return (y * pow2i(m - 1)) * 2.0;  // just below the overflow threshold
  if (m >= -1020) return y * pow2i(m);
  return (y * pow2i(m + 54)) * 0x1p-54;  // result subnormal: scale in two steps
}

}  // namespace ecpgb

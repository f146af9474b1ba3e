// ecp_fastmath.h -- FP64 exp for the batched path (host and device).
//
// Table-driven method of P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15 (1989)
// 144-157, written here from that description:
//   x = (32 m + j) ln2/32 + r,  |r| <= ln2/64,
//   exp(x) = 2^m * 2^(j/32) * exp(r),
// with exp(r) - 1 from its degree-6 Taylor polynomial (truncation below
// 4e-18 relative on |r| <= ln2/64), the 32 values 2^(j/32) rounded to
// nearest (computed to 60 digits), and the reduction done with a two-part
// ln2/32 whose leading part has 31 significant bits, so n * L1 is exact.
// Maximum error about 1.5 ulp; tests/test_fastmath.py measures it against
// the C library's exp.  About 12 FP64 operations against ~24 for a general
// exp, which matters on GB300 where FP64 runs at 1/62 of the FP32 rate.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define ECPGB_HD __host__ __device__ __forceinline__
#else
#define ECPGB_HD inline
#endif

namespace ecpgb {

#define ECPGB_EXP2_32                                                                                    \
  {0x1.0000000000000p+0, 0x1.059b0d3158574p+0, 0x1.0b5586cf9890fp+0, 0x1.11301d0125b51p+0,              \
   0x1.172b83c7d517bp+0, 0x1.1d4873168b9aap+0, 0x1.2387a6e756238p+0, 0x1.29e9df51fdee1p+0,              \
   0x1.306fe0a31b715p+0, 0x1.371a7373aa9cbp+0, 0x1.3dea64c123422p+0, 0x1.44e086061892dp+0,              \
   0x1.4bfdad5362a27p+0, 0x1.5342b569d4f82p+0, 0x1.5ab07dd485429p+0, 0x1.6247eb03a5585p+0,              \
   0x1.6a09e667f3bcdp+0, 0x1.71f75e8ec5f74p+0, 0x1.7a11473eb0187p+0, 0x1.82589994cce13p+0,              \
   0x1.8ace5422aa0dbp+0, 0x1.93737b0cdc5e5p+0, 0x1.9c49182a3f090p+0, 0x1.a5503b23e255dp+0,              \
   0x1.ae89f995ad3adp+0, 0x1.b7f76f2fb5e47p+0, 0x1.c199bdd85529cp+0, 0x1.cb720dcef9069p+0,              \
   0x1.d5818dcfba487p+0, 0x1.dfc97337b9b5fp+0, 0x1.ea4afa2a490dap+0, 0x1.f50765b6e4540p+0}

#ifdef __CUDACC__
static __device__ const double kExp2Table32Dev[32] = ECPGB_EXP2_32;
#endif
static const double kExp2Table32Host[32] = ECPGB_EXP2_32;

ECPGB_HD double pow2i(int m) {  // 2^m for -1022 <= m <= 1023
  long long bits = (long long)(m + 1023) << 52;
  double d;
#ifdef __CUDA_ARCH__
  d = __longlong_as_double(bits);
#else
  std::memcpy(&d, &bits, sizeof d);
#endif
  return d;
}

ECPGB_HD double fast_exp(double x) {
  const double inv = 0x1.71547652b82fep+5;   // 32 / ln2
  const double L1 = 0x1.62e42fee00000p-6;    // ln2/32, leading 31 bits
  const double L2 = 0x1.a39ef35793c76p-38;   // ln2/32 - L1
  if (!(x > -745.2)) return (x != x) ? x : 0.0;  // NaN stays NaN, underflow to 0
  if (x > 709.78) return HUGE_VAL;
  double t = std::rint(x * inv);
  int n = (int)t;
  double r = std::fma(-t, L1, x);
  r = std::fma(-t, L2, r);
  int j = n & 31, m = (n - j) / 32;
  double p = std::fma(r, 1.0 / 720.0, 1.0 / 120.0);
  p = std::fma(p, r, 1.0 / 24.0);
  p = std::fma(p, r, 1.0 / 6.0);
  p = std::fma(p, r, 0.5);
  p = std::fma(p, r, 1.0);
  p = p * r;  // exp(r) - 1
#ifdef __CUDA_ARCH__
  const double s = kExp2Table32Dev[j];
#else
  const double s = kExp2Table32Host[j];
#endif
  double y = std::fma(s, p, s);
  if (m >= -1020) return y * pow2i(m);
  return (y * pow2i(m + 54)) * 0x1p-54;  // result subnormal: scale in two steps
}

}  // namespace ecpgb

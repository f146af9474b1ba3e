// ecp_ff.h -- double-single ("ff") arithmetic for the mixed-precision path.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)
// (about 48 significant bits).  The algorithms are the error-free
// transformations of Dekker and Knuth (two-sum, fast two-sum) and the
// FMA-based exact product (two-prod), combined as in Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44 (2017).  Every operation is an FP32
// add, multiply or FMA, so on GB300 the work runs on the FMA pipes (128
// lanes per SM and cycle) instead of the FP64 pipe (2 lanes per SM and
// cycle).  The header compiles for the host as well, where the same
// operations give the same results, so the CPU tests check it.
//
// Range: floats.  The mixed path uses ff only for quantities bounded by
// their screens (Gaussian exponents >= ln(1e-14) - 2, K_l(z) <= 1, ECP terms
// with a r^2 <= 87), so values below ~1e-31 of the largest term of a sum may
// lose precision or flush to zero; their contribution is below the parity bar
// by many orders of magnitude.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "ecp_exp2_table.h"

#ifdef __CUDACC__
#define FF_HD __host__ __device__ __forceinline__
#else
#define FF_HD inline
#endif

namespace ecpgb {

struct ff {
  float hi, lo;
};

FF_HD float ff_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
// plain FP32 operations that must not be contracted into FMAs (on the host
// the tests compile with -ffp-contract=off)
FF_HD float f_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
FF_HD float f_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

// s + t = a + b exactly, |a| >= |b| (or a == 0)
FF_HD ff fast_two_sum(float a, float b) {
  const float s = f_add(a, b);
  return {s, f_add(b, -f_add(s, -a))};
}
// s + t = a + b exactly, any order
FF_HD ff two_sum(float a, float b) {
  const float s = f_add(a, b);
  const float bb = f_add(s, -a);
  const float aa = f_add(s, -bb);
  return {s, f_add(f_add(a, -aa), f_add(b, -bb))};
}
// p + e = a * b exactly
FF_HD ff two_prod(float a, float b) {
  const float p = f_mul(a, b);
  return {p, ff_fma(a, b, -p)};
}

FF_HD ff ff_norm(float hi, float lo) { return fast_two_sum(hi, lo); }  // |lo| small against |hi|

// 2^m as a float, -126 <= m <= 127
FF_HD float pow2f(int m) {
  const uint32_t b = (uint32_t)(m + 127) << 23;
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, 4);
  return f;
#endif
}

FF_HD ff ff_from_float(float a) { return {a, 0.0f}; }

// ff + ff (accurate: both operands' errors, any signs)
FF_HD ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  float c = f_add(s.lo, t.hi);
  ff v = ff_norm(s.hi, c);
  float w = f_add(t.lo, v.lo);
  return ff_norm(v.hi, w);
}
// ff + ff where the operands do not cancel (same sign, or |b| << |a|)
FF_HD ff ff_add_sloppy(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  return ff_norm(s.hi, f_add(s.lo, f_add(a.lo, b.lo)));
}
FF_HD ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
// ff * ff
FF_HD ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  float e = ff_fma(a.hi, b.lo, p.lo);
  e = ff_fma(a.lo, b.hi, e);
  return ff_norm(p.hi, e);
}
// ff * float
FF_HD ff ff_mul_f(ff a, float b) {
  ff p = two_prod(a.hi, b);
  return ff_norm(p.hi, ff_fma(a.lo, b, p.lo));
}

// A double split into ff (hi = the nearest float, lo = the nearest float to
// the remainder).  Host side, or once per primitive pair on the device.
FF_HD ff ff_from_double(double d) {
  const float hi = (float)d;
  if (!std::isfinite(hi)) return {hi, 0.0f};
  return {hi, (float)(d - (double)hi)};
}
FF_HD double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// Compensated running sum (Ogita, Rump and Oishi's Sum2): the terms are
// added with two-sum, their rounding errors collected in a second float.
struct ff_acc {
  float s = 0.0f, c = 0.0f;
  FF_HD void add(ff x) {
    ff t = two_sum(s, x.hi);
    s = t.hi;
    c = f_add(c, f_add(t.lo, x.lo));
  }
  FF_HD double value() const { return (double)s + (double)c; }
};

// 2^(j/512) as ff, from the FP64 table of ecp_exp2_table.h.
struct Exp2TableFF {
  float hi[ECPGB_EXP2_N], lo[ECPGB_EXP2_N];
  constexpr Exp2TableFF() : hi(), lo() {
    constexpr double t[ECPGB_EXP2_N] = ECPGB_EXP2_TABLE;
    for (int j = 0; j < ECPGB_EXP2_N; j++) {
      hi[j] = (float)t[j];
      lo[j] = (float)(t[j] - (double)hi[j]);
    }
  }
};
#ifdef __CUDACC__
static __device__ const Exp2TableFF kExp2FFDev;
#endif
static const Exp2TableFF kExp2FFHost;

// ln2 / 512 as the sum of three floats (each the nearest float to what the
// previous ones leave; generated with 300-bit arithmetic, residual 6e-27),
// and 512 / ln2 rounded to a float.
constexpr float kL1 = 0x1.62e43p-10f;
constexpr float kL2 = -0x1.05c61p-38f;
constexpr float kL3 = -0x1.950d88p-63f;
constexpr float kInvL = 0x1.715476p+9f;

// exp(x) for x in ff, written from Tang's table-driven method (ACM TOMS 15
// (1989) 144): x = k ln2/512 + r, exp(x) = 2^(k >> 9) 2^((k & 511)/512)
// exp(r).  The reduction is done exactly with two-prod on the two leading
// pieces of ln2/512 (x and k ln2/512 agree to a factor of two, so their
// difference is exact by Sterbenz's lemma), exp(r) - 1 by its Taylor
// polynomial to r^4 (truncation below 2^-50 for |r| <= ln2/1024), the
// high-order part in plain FP32.  Results below 2^-126 are returned as 0;
// the arguments here are <= 0 or small.  Relative error about 2^-46 where the
// result is above 2^-100 (x > -69); below that its low part leaves the float
// range and the absolute error stays below 2^-140 (tests/test_ff.py).
FF_HD ff ff_exp(ff x) {
  if (x.hi < -87.0f) return {0.0f, 0.0f};
  const float k = rintf(f_mul(x.hi, kInvL));
  const ff p1 = two_prod(k, kL1);
  const float t = f_add(x.hi, -p1.hi);  // exact (Sterbenz)
  ff r = two_sum(t, -p1.lo);
  r = ff_norm(r.hi, f_add(r.lo, x.lo));
  const ff p2 = two_prod(k, kL2);
  r = ff_add(r, {-p2.hi, -p2.lo});
  r = ff_norm(r.hi, f_add(r.lo, -f_mul(k, kL3)));
  // exp(r) - 1 = r + r^2 / 2 + r^2 d, d = r / 6 + r^2 / 24: r^2 / 2 exactly
  // in ff, the r^2 d term (below 2^-34) in FP32
  const float d = f_mul(ff_fma(r.hi, 1.0f / 24.0f, 1.0f / 6.0f), r.hi);
  ff r2 = two_prod(r.hi, r.hi);
  const float r2lo = ff_fma(2.0f * r.hi, r.lo, r2.lo);
  const ff half = ff_norm(0.5f * r2.hi, ff_fma(r2.hi, d, 0.5f * r2lo));
  const ff poly = ff_add_sloppy(r, half);
  const int ki = (int)k, j = ki & (ECPGB_EXP2_N - 1), m = (ki - j) / ECPGB_EXP2_N;
#ifdef __CUDA_ARCH__
  const ff T = {kExp2FFDev.hi[j], kExp2FFDev.lo[j]};
#else
  const ff T = {kExp2FFHost.hi[j], kExp2FFHost.lo[j]};
#endif
  const ff y = ff_add_sloppy(T, ff_mul(T, poly));
  if (m < -126) return {0.0f, 0.0f};
  const float sc = pow2f(m);
  return {f_mul(y.hi, sc), f_mul(y.lo, sc)};
}

}  // namespace ecpgb

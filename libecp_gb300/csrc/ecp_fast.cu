// ecp_fast.cu -- batched unit kernel for sm_103a (the fast FP64 path).
//
// Same results as the drop-in kernel (same quadrature schedules, windows,
// convergence tests, stale-buffer semantics of the reference's fallbacks);
// the work is organised for GB300, where FP64 runs at 1/62 of the FP32 rate
// and every FP64 operation counts:
//   * a warp per primitive pair (pairs dealt round-robin to the 4 warps):
//     no CTA barrier inside the type-1 loop or the type-2 fallback;
//   * level-granular tabulation: grid points are tabulated 32 schedule slots
//     at a time (one slot per lane) and a primitive pair stops as soon as all
//     its quadratures have converged -- on the 50-centre cluster the type-2
//     fallback's quadratures stop after ~280 of the 1023 large-grid slots,
//     where the reference tabulates all 1023;
//   * K_l(z) as one Horner pass over precomputed Taylor coefficients (the
//     reference's 5-step derivative recurrence, done once per table point on
//     the host); exp by the table-driven method of ecp_fastmath.h; no FP64
//     divide or trigonometric call in the hot loops (tabulated abscissae and
//     reciprocals, division-free convergence tests, the k-vector direction
//     from ratios);
//   * only what is read is computed: type-1 tabulation for the pairs with a
//     quadrature still running, fallback rows for the quadratures still
//     running, and in the type-2 fallback only the slots whose value passes
//     the screen (a pair's own points through its index interval), walked
//     pair by pair with the empty slot pairs skipped;
//   * the type-1 block accumulated per combined Cartesian index: chi[i][j]
//     depends on (i, j) only through the index of a_i + b_j
//     (src/type1.c:323-345), so one accumulator per combined index receives
//     exactly the terms the reference adds to each chi[i][j];
//   * the precision mode a template parameter: the FP64 kernels carry no
//     mixed-precision code (instruction fetch is one of the kernel's stalls).
#include "ecp_device.cuh"
#include "ecp_fastmath.h"

namespace ecpgb {

constexpr int kWarps = kUnitThreads / 32;
// CTAs per SM the unit kernels are compiled for (168 registers a thread):
// with the target stated, the register allocator keeps the spills to a few
// bytes (without it: 168 registers and 0.8 KB of spill traffic a thread)
constexpr int kUnitCtasPerSm = 3;
constexpr int kWalkCap = 128;  // large-grid quadratures per warp and pass
constexpr int kLargeWords = (kMaxLargeOrder + 1) / 32;  // bitmap words over the large grid (128, even)
static_assert(kLargeWords * 32 >= kMaxLargeOrder && kLargeWords % 2 == 0, "large-grid bitmap size");


// --------------------------------------------------------------- helpers

// K_0..K_lmax(z): the branches of src/bessel.c:102-199.  The Taylor branch
// (z < 16) and the large-argument branch are both one Horner pass per row, in
// dz over the row's Taylor coefficients or in -1/(2z) over the row's
// large-argument polynomial, so that lanes on either branch run the same
// instructions: row l is a polynomial of degree max(5, l) whose coefficients
// above the branch's own degree are zero.
// K_0..K_lmax(z) for z < 1e-7: the reference's zeroth-order branch,
// K_l = (1 - z) z^l / (2l+1)!! by its recurrence (src/bessel.c:118-133).
static __device__ void bessel_small(int lmax, double z, double *K, int stride) {
  if (z <= 0) {
    K[0] = 1.0;
    for (int l = 1; l <= lmax; l++) K[l * stride] = 0.0;
  } else {
    K[0] = 1 - z;
    for (int l = 1; l <= lmax; l++) K[l * stride] = K[(l - 1) * stride] * z / (2 * l + 1);
  }
}

template <bool kMixed>
static __device__ __noinline__ void bessel_fast(const DevJob &J, int lmax, double z, double *K, int stride) {
  if (__builtin_expect(z < 1.0E-7, 0)) {  // rare: laid out of line
    bessel_small(lmax, z, K, stride);
    return;
  }
  const bool asy = z >= 16.0;
  const int HL1 = J.besHL + 1;
  double x, mult = 1.0;
  const double *cf;
  int cs;
  if (asy) {
    mult = 0.5 * __drcp_rn(z);  // = 0.5 / z exactly (scaling by 2^-1)
    x = -mult;
    cf = J.besA;
    cs = HL1 < 6 ? 6 : HL1;
  } else {
    const double h = J.besselN / 16;  // integer division, as the reference
    const int index = (int)floor(z * h + 0.5);
    x = z - __ldg(J.besZ + index);  // index / h, tabulated
    cf = J.besH + (size_t)index * HL1 * 6;
    cs = 6;
  }
  for (int l = 0; l <= lmax; l++) {
    const double *q = cf + l * cs;
    // Horner from the row's top coefficient (degree l on the large-argument
    // branch above 5, else 5): no multiply of a zero, no scaling by 1
    int k = asy && l > 5 ? l : 5;
    double v = q[k];
    while (k > 5) {
      k--;
      v = fma(v, x, q[k]);
    }
#pragma unroll
    for (int j = 4; j >= 0; j--) v = fma(v, x, q[j]);
    if (asy) v *= mult;
    K[l * stride] = v;
  }
}

// One row K_l(z), by the same branches as bessel_fast.
static __device__ __noinline__ double bessel_row(const DevJob &J, int l, double z) {
  if (__builtin_expect(z < 1.0E-7, 0)) {  // rare: laid out of line
    if (z <= 0) return l == 0 ? 1.0 : 0.0;
    double v = 1 - z;
    for (int i = 1; i <= l; i++) v = v * z / (2 * i + 1);
    return v;
  }
  if (z >= 16.0) {
    const int HL1 = J.besHL + 1;
    const double mult = 0.5 * __drcp_rn(z), x = -mult;
    const double *q = J.besA + (size_t)l * (HL1 < 6 ? 6 : HL1);
    int k = l > 5 ? l : 5;
    double v = q[k];
    while (k > 0) {
      k--;
      v = fma(v, x, q[k]);
    }
    return v * mult;
  }
  double h = J.besselN / 16;
  int index = (int)floor(z * h + 0.5);
  double dz = z - __ldg(J.besZ + index);  // index / h, tabulated
  const double *q = J.besH + ((size_t)index * (J.besHL + 1) + l) * 6;
  double v = fma(q[5], dz, q[4]);
  v = fma(v, dz, q[3]);
  v = fma(v, dz, q[2]);
  v = fma(v, dz, q[1]);
  return fma(v, dz, q[0]);
}

// U_l(r) of centre c for the channels l set in mask, in one pass over its
// terms (src/ecp.c:42-60); the other entries of U are left untouched.
template <bool kMixed>
static __device__ __noinline__ void channels_masked(const DevJob &J, int c, double r, unsigned mask, double *U) {
  double r2 = r * r;
  for (unsigned m = mask; m; m &= m - 1) U[__ffs(m) - 1] = 0.0;
  int t0 = J.ctrT0[c], t1 = t0 + J.ctrNT[c];
  for (int t = t0; t < t1; t++) {
    int l = J.termL[t];
    if (mask >> l & 1u) U[l] += rpow(r, J.termN[t]) * J.termD[t] * fast_exp(-J.termA[t] * r2);
  }
}

template <bool kMixed>
static __device__ __noinline__ double channel(const DevJob &J, int c, int l, double r) {
  double r2 = r * r, pot = 0.0;
  int t0 = J.ctrT0[c], t1 = t0 + J.ctrNT[c];
  for (int t = t0; t < t1; t++)
    if (J.termL[t] == l) pot += rpow(r, J.termN[t]) * J.termD[t] * fast_exp(-J.termA[t] * r2);
  return pot;
}

// ------------------------------------------- double-single (mixed path)
//
// The mixed path evaluates the large-grid fallbacks' tables -- Bessel rows,
// ECP channels, powers of r, the Gaussian prefactor -- and their integrand
// products in double-single arithmetic (ecp_ff.h: FP32 pairs on the FMA
// pipes), sums each level of a quadrature with a compensated FP32 sum and
// adds it to the FP64 running sum at the level's end.  The convergence
// tests, the level recurrences and every accumulation into T, Q and the
// blocks stay FP64.  The fallbacks' test (PSM92, 16 e^2 <= 3 N |I - q| tol)
// compares level differences far above the double-single rounding, so it
// takes the FP64 path's decisions; the small-grid quadratures, whose
// absolute test (err < tol) sits at the FP64 rounding level for large
// integrals, are not touched.

// 1 / z: the float reciprocal refined by one Newton step in ff.
static __device__ inline ff ff_recip(ff z) {
  const float y = __frcp_rn(z.hi);
  const float e = __fmaf_rn(-z.lo, y, __fmaf_rn(-z.hi, y, 1.0f));  // 1 - z y
  return ff_norm(y, __fmul_rn(y, e));
}

// K_0..K_lmax(z) in ff: the branches of bessel_fast over the tables' float
// pairs (Taylor coefficients, table abscissae, large-argument polynomial).
static __device__ __noinline__ void bessel_ff(const DevJob &J, int lmax, ff z, ff *K, int stride) {
  if (__builtin_expect(z.hi < 1.0e-7f, 0)) {  // rare: the small-argument formula in FP64
    double Kd[kMaxRows];
    bessel_small(lmax, ff_to_double(z), Kd, 1);
    for (int l = 0; l <= lmax; l++) K[l * stride] = ff_from_double(Kd[l]);
    return;
  }
  const int HL1 = J.besHL + 1;
  if (z.hi > 16.0f || (z.hi == 16.0f && z.lo >= 0.0f)) {
    const ff inv = ff_recip(z);
    const ff mult = {0.5f * inv.hi, 0.5f * inv.lo}, x = ff_neg(mult);  // 1/(2z), -1/(2z)
    const int cs = HL1 < 6 ? 6 : HL1;
    for (int l = 0; l <= lmax; l++) {
      const ff *q = J.besAf + (size_t)l * cs;
      int k = l > 5 ? l : 5;
      ff v = q[k];
      while (k > 0) {
        k--;
        v = ff_add(ff_mul(v, x), q[k]);
      }
      K[l * stride] = ff_mul(v, mult);
    }
    return;
  }
  // the nearest table point; any neighbour would do as well (the Taylor
  // series is accurate over the whole table step)
  const int index = (int)floorf(__fmaf_rn(z.hi, (float)(J.besselN / 16), 0.5f));
  const ff x = ff_add(z, ff_neg(J.besZf[index]));
  const ff *qf = J.besHf + (size_t)index * HL1 * 6;
  for (int l = 0; l <= lmax; l++) {
    const ff *q = qf + 6 * l;
    // the two top terms (below 1e-9 of the row) in FP32
    ff v = ff_add(ff_mul_f(x, __fmaf_rn(q[5].hi, x.hi, q[4].hi)), q[3]);
    v = ff_add(ff_mul(v, x), q[2]);
    v = ff_add(ff_mul(v, x), q[1]);
    K[l * stride] = ff_add(ff_mul(v, x), q[0]);
  }
}

// One ECP term d r^n exp(-a r^2) in ff (r2 = r^2); terms below 2^-125 of
// their coefficient are 0.
static __device__ inline ff ecp_term_ff(const DevJob &J, int t, ff r, ff r2) {
  const ff arg = ff_mul(J.termAf[t], r2);
  if (arg.hi > 87.0f) return {0.0f, 0.0f};
  const ff v = ff_mul(J.termDf[t], ff_exp(ff_neg(arg)));
  const double n = J.termN[t];
  if (n == 0.0) return v;
  if (n == 1.0) return ff_mul(v, r);
  if (n == 2.0) return ff_mul(v, r2);
  return ff_mul(v, ff_from_double(rpow(ff_to_double(r), n)));  // other powers: rare
}

// U_l(r) in ff for the channels set in mask (the others untouched).
static __device__ __noinline__ void channels_ff(const DevJob &J, int c, ff r, unsigned mask, ff *U) {
  const ff r2 = ff_mul(r, r);
  for (unsigned m = mask; m; m &= m - 1) U[__ffs(m) - 1] = {0.0f, 0.0f};
  const int t0 = J.ctrT0[c], t1 = t0 + J.ctrNT[c];
  for (int t = t0; t < t1; t++) {
    const int l = J.termL[t];
    if (mask >> l & 1u) U[l] = ff_add(U[l], ecp_term_ff(J, t, r, r2));
  }
}

static __device__ __noinline__ ff channel_ff(const DevJob &J, int c, int l, ff r) {
  const ff r2 = ff_mul(r, r);
  ff pot = {0.0f, 0.0f};
  const int t0 = J.ctrT0[c], t1 = t0 + J.ctrNT[c];
  for (int t = t0; t < t1; t++)
    if (J.termL[t] == l) pot = ff_add(pot, ecp_term_ff(J, t, r, r2));
  return pot;
}

// Small-grid prefactor of a type-1 primitive pair, C1 = ca cb exp(zd2) with
// zd2 = -za dAC^2 - zb dBC^2 (src/type1.c:235-246), rounded as the reference
// rounds it (no contraction), so that every evaluation of it agrees.
static __device__ inline double t1_prefactor(double za, double ca, double zb, double cb, double dAC, double dBC) {
  const double zd2 = __dsub_rn(__dmul_rn(__dmul_rn(-za, dAC), dAC), __dmul_rn(__dmul_rn(zb, dBC), dBC));
  return __dmul_rn(__dmul_rn(ca, cb), fast_exp(zd2));
}

// Kinds of type-1 primitive pairs.  The reference's small-grid integrand is
// C1 r^l U K exp(e), e = (z r + s) r, multiplied left to right
// (src/type1.c:79-88).
//  * normal: C1 >= 2^-900 and e <= s^2 / (4 (za + zb)) < 700: no partial
//    product of a non-negligible term underflows and exp(e) cannot overflow,
//    so the integrand can be regrouped (prefactor, weight and r^l in one
//    table row);
//  * band: C1 below 2^-900 but not 0, or exp(e) may overflow: partial
//    products underflow (or overflow) where a regrouped product would not, so
//    the integrand is evaluated in the reference's order;
//  * zero: C1 = 0, so every integrand value is 0 * (finite) = 0, or NaN where
//    exp(e) overflows -- no table is needed.
constexpr int kPairNormal = 0, kPairBand = 1, kPairZero = 2;
constexpr double kLnDblMax = 0x1.62e42fefa39efp+9;  // exp overflows above it

// e = (z r + s) r as the reference rounds it.
static __device__ inline double t1_exponent(double z, double s, double r) {
  return __dmul_rn(__dadd_rn(__dmul_rn(z, r), s), r);
}

// A zero-kind pair's PS93 walk (src/gc_integrators.c:157-217) with an
// integrand that is 0 except NaN at window points whose exp(e) overflows:
// the first level that counts a point converges to 0 unless a NaN has been
// summed by then, after which no level converges.
static __device__ __noinline__ bool t1_zero_walk(const DevJob &J, double s, double z, int ws, int we) {
  auto nan_at = [&](int n) {
    if (n < ws || n >= we) return false;
    const double e = t1_exponent(z, s, J.xSmall[n]);
    return e >= J.lnAcc1 && e > kLnDblMax;
  };
  bool nan = nan_at(c93_slot[0]) || nan_at(c93_slot[1]) || nan_at(c93_slot[2]);
  int pos = 3;
  for (int k = 0; k < c93_nLevels; k++) {
    const int e = c93_lvEnd[k];
    int cnt = 0;
    for (; pos < e; pos += 2) {
      const int lo = c93_slot[pos], hi = c93_slot[pos + 1];
      if (lo >= ws) { nan = nan || nan_at(lo); cnt++; }
      if (hi <= we) { nan = nan || nan_at(hi); cnt++; }
    }
    if (cnt > 0) return !nan;
  }
  return false;
}

// FM06 map parameters (src/gc_integrators.c:317-331).
static __device__ inline void fm06(double za, double zb, double dAC, double dBC, double &i1, double &i2) {
  double zp = za + zb, P = (za * dAC + zb * dBC) / zp;
  double sigma = 1.0 / sqrt(zp), t = P - 7.0 * sigma;
  double rmin = (t > 0.0) ? t : 0.0, rmax = P + 9.0 * sigma;
  i1 = 0.5 * (rmax - rmin);
  i2 = 0.5 * (rmax + rmin);
}

// Schedule steps: step 0 = the head plus 15 (lower, upper) pairs, every later
// step 16 pairs.  For the large grid step 0 ends exactly at level 3.
static __device__ inline int step_end93(int s0) { return s0 == 0 ? 33 : s0 + 32; }
static __device__ inline int step_end92(int s0) { return s0 == 0 ? 31 : s0 + 32; }

// PSM92 walker (src/gc_integrators.c:39-86) over slots [s0, s1) of the
// large-grid schedule; `val(pos)` = w * f at slot pos; `vis(pos)` whether the
// (upper) point counts.  State in I, p, q; returns through done/res.
template <class V, class Vis>
static __device__ inline void psm92_advance(int s0, int s1, double tol, V val, Vis vis,
                                            double &I, double &p, double &q, bool &done, double &res) {
  int pos = s0;
  if (pos == 0) {
    I = val(0);
    p = I;
    pos = 1;
  }
  int k = level_of(pos);
  while (pos < s1 && !done) {
    int lvStart = k == 0 ? 1 : c92_lvEnd[k - 1];
    if (pos == lvStart) {
      q = 2 * p;
      p = 2 * I;
    }
    double T = 0.0;
    T += val(pos);
    if (vis(pos + 1)) T += val(pos + 1);
    I += T;
    pos += 2;
    if (pos == c92_lvEnd[k]) {
      double N = c92_lvN[k] + 1.0, e = I - p;
      if (16 * e * e <= 3 * N * fabs(I - q) * tol) {
        res = 16 * I / (3 * N);
        done = true;
      }
      k++;
    }
  }
}

// PS93 walk of ps93_walk (src/gc_integrators.c:157-217) with the error test
// 16 d / (3 n) < tol written as 16 d < tol 3 n: no divide per level (the
// same decision but within an ulp of the threshold).
template <class Fn>
static __device__ bool ps93_walk_fast(const double *w, int start, int end, double tol, Fn f, double &res) {
  int mid = c93_slot[0], a = c93_slot[1], b = c93_slot[2];
  double p = w[mid] * f(mid);
  double q = w[a] * f(a) + w[b] * f(b);
  double I = p + q;
  int pos = 3;
  for (int k = 0; k < c93_nLevels; k++) {
    int j = c93_lvJ[k], cnt = 0, e = c93_lvEnd[k];
    for (; pos < e; pos += 2) {
      int lo = c93_slot[pos], hi = c93_slot[pos + 1];
      double T = 0.0;
      if (lo >= start) { T += w[lo] * f(lo); cnt++; }
      if (hi <= end) { T += w[hi] * f(hi); cnt++; }
      I += T;
    }
    int n = c93_lvN[k];
    p += (1 - j) * (I - q);
    const double d = fabs((1 - j) * (q - 3 * p / 2) + j * (I - 2 * q));
    q = (1 - j) * q + j * I;
    if (cnt == 0) continue;
    if (16 * d < tol * (3 * n)) {
      res = 16 * q / (3 * n);
      return true;
    }
  }
  res = 16 * q / (3 * c93_lvN[c93_nLevels - 1]);  // the last estimate (mixed path: its size)
  return false;
}

// psm92_advance over the slots [s0, s1) whose bit is set in `bits`; the
// other slots integrate to exactly zero, so (lower, upper) pairs without a set
// bit are skipped -- adding 0.0 changes no sum -- while every level end is
// still visited in order for the convergence test.
template <class V, class Vis>
static __device__ inline void psm92_sparse(int s0, int s1, const unsigned *bits, double tol, V val,
                                           Vis vis, double &I, double &p, double &q, bool &done, double &res) {
  auto has = [&](int t) { return (bits[t >> 5] >> (t & 31)) & 1u; };
  int pos = s0;
  if (pos == 0) {
    I = has(0) ? val(0) : 0.0;
    p = I;
    pos = 1;
  }
  int k = level_of(pos);
  while (pos < s1 && !done) {
    const int lvStart = k == 0 ? 1 : c92_lvEnd[k - 1];
    if (pos == lvStart) {
      q = 2 * p;
      p = 2 * I;
    }
    const int lvE = c92_lvEnd[k], stop = lvE < s1 ? lvE : s1;
    while (true) {
      int t = stop;  // first set bit in [pos, stop)
      for (int w = pos >> 5; (w << 5) < stop; w++) {
        unsigned word = bits[w];
        if (w == (pos >> 5)) word &= ~0u << (pos & 31);
        if (word) {
          t = (w << 5) + __ffs(word) - 1;
          break;
        }
      }
      if (t >= stop) {
        pos = stop;
        break;
      }
      const int ps = (t - 1) | 1;  // the (lower, upper) pair holding t
      double T = 0.0;
      if (has(ps)) T += val(ps);
      if (has(ps + 1) && vis(ps + 1)) T += val(ps + 1);
      I += T;
      pos = ps + 2;
    }
    if (pos == lvE) {
      double N = c92_lvN[k] + 1.0, e = I - p;
      if (16 * e * e <= 3 * N * fabs(I - q) * tol) {
        res = 16 * I / (3 * N);
        done = true;
      }
      k++;
    }
  }
}

// psm92_advance with val(pos) in ff: each level summed with a compensated
// FP32 sum and added to the FP64 running sum I at the level's end (and at
// the end of the slots walked, so that I is complete between calls).
template <class V, class Vis>
static __device__ inline void psm92_advance_ff(int s0, int s1, double tol, V val, Vis vis, double &I, double &p,
                                               double &q, bool &done, double &res) {
  int pos = s0;
  if (pos == 0) {
    I = ff_to_double(val(0));
    p = I;
    pos = 1;
  }
  int k = level_of(pos);
  ff_acc acc;
  while (pos < s1 && !done) {
    int lvStart = k == 0 ? 1 : c92_lvEnd[k - 1];
    if (pos == lvStart) {
      q = 2 * p;
      p = 2 * I;
    }
    acc.add(val(pos));
    if (vis(pos + 1)) acc.add(val(pos + 1));
    pos += 2;
    if (pos == c92_lvEnd[k]) {
      I += acc.value();
      acc = ff_acc();
      double N = c92_lvN[k] + 1.0, e = I - p;
      if (16 * e * e <= 3 * N * fabs(I - q) * tol) {
        res = 16 * I / (3 * N);
        done = true;
      }
      k++;
    }
  }
  I += acc.value();
}

// psm92_sparse with val(pos) in ff, levels summed as in psm92_advance_ff.
template <class V, class Vis>
static __device__ inline void psm92_sparse_ff(int s0, int s1, const unsigned *bits, double tol, V val, Vis vis,
                                              double &I, double &p, double &q, bool &done, double &res) {
  auto has = [&](int t) { return (bits[t >> 5] >> (t & 31)) & 1u; };
  int pos = s0;
  if (pos == 0) {
    I = has(0) ? ff_to_double(val(0)) : 0.0;
    p = I;
    pos = 1;
  }
  int k = level_of(pos);
  ff_acc acc;
  while (pos < s1 && !done) {
    const int lvStart = k == 0 ? 1 : c92_lvEnd[k - 1];
    if (pos == lvStart) {
      q = 2 * p;
      p = 2 * I;
    }
    const int lvE = c92_lvEnd[k], stop = lvE < s1 ? lvE : s1;
    while (true) {
      int t = stop;  // first set bit in [pos, stop)
      for (int w = pos >> 5; (w << 5) < stop; w++) {
        unsigned word = bits[w];
        if (w == (pos >> 5)) word &= ~0u << (pos & 31);
        if (word) {
          t = (w << 5) + __ffs(word) - 1;
          break;
        }
      }
      if (t >= stop) {
        pos = stop;
        break;
      }
      const int ps = (t - 1) | 1;  // the (lower, upper) pair holding t
      if (has(ps)) acc.add(val(ps));
      if (has(ps + 1) && vis(ps + 1)) acc.add(val(ps + 1));
      pos = ps + 2;
    }
    if (pos == lvE) {
      I += acc.value();
      acc = ff_acc();
      double N = c92_lvN[k] + 1.0, e = I - p;
      if (16 * e * e <= 3 * N * fabs(I - q) * tol) {
        res = 16 * I / (3 * N);
        done = true;
      }
      k++;
    }
  }
  I += acc.value();
}

// --------------------------------------------------------------- layout

// Quadratures per primitive pair in the type-1 block ((l1, l2), l2 = l1,
// l1-2, ...; src/type1.c:189-202), and primitive pairs packed per warp so
// that most lanes carry a quadrature.
__host__ __device__ inline int t1_items(int lab) {
  int n = 0;
  for (int l1 = 0; l1 <= lab; l1++) n += l1 / 2 + 1;
  return n;
}
__host__ __device__ inline int t1_group(int lab, int cap) {
  int g = 32 / t1_items(lab);
  g = g > 8 ? 8 : (g < 1 ? 1 : g);
  // the group's step table (33 slots x g entries of 2 (lab+1) + 1 doubles)
  // stays within 33 x cap doubles (cap 45: three CTAs per SM at l <= 3, L <= 4)
  while (g > 1 && g * (2 * lab + 3) > cap) g--;
  return g;
}

struct FastSmem {
  int chi, J, T, phase, total;
  // type-1 per warp (inside phase): pair scalars, S_lm, Q, H, step table
  int w1Stride, w1Sc, w1Rsh, w1Q, w1H, w1Tab;
  // type-2 fallback per warp (inside phase)
  int w2Stride, w2Tab, w2I, w2P, w2Q, w2R, w2Part, tab2Stride;
  int w2Bits, w2Pend, w2Pref;  // fallback streaming: needed-slot bitmap, pending slots, word prefixes
  int ppMap;                   // type-2 fallback: FM06 map (i1, i2) of every primitive pair
  int ppWin;                   // and the point-index interval where its exponent can pass the screen
};

__host__ __device__ inline FastSmem fast_layout(int LB, int LE, int cap, int maxNP) {
  FastSmem s{};
  const int nA = 2 * LB + 1, nE = LE > 0 ? LE : 1, LBE = LB + nE;
  const int nc = (LB + 1) * (LB + 2) * (LB + 3) / 6, nct = (LB + 1) * (LB + 2) / 2;
  const int ncAB = (2 * LB + 1) * (2 * LB + 2) * (2 * LB + 3) / 6;
  int rq = 0, tt = 0;  // largest per-warp S_lm/Q and step-table widths over lab <= 2 LB
  for (int lab = 0; lab <= 2 * LB; lab++) {
    int g = t1_group(lab, cap), lq = lab + 1;
    if (g * lq * lq > rq) rq = g * lq * lq;
    // small-grid steps: 33 slots x g entries of 2 lq + 1; fallback steps: 32
    // slots of 2 lq + 3
    if (33 * g * (1 + 2 * lq) > tt) tt = 33 * g * (1 + 2 * lq);
    if (32 * (3 + 2 * lq) > tt) tt = 32 * (3 + 2 * lq);
  }
  int o = 0;
  s.chi = o; o += nc * nc;
  s.J = o; o += nct * nc;
  s.T = o; o += nE * LBE * LBE * nA;
  s.phase = o;
  s.w1Sc = 0;
  s.w1Rsh = 48;  // pair scalars: 6 per pair, up to 8 pairs
  s.w1Q = s.w1Rsh + rq;
  s.w1H = s.w1Q + rq;
  s.w1Tab = s.w1H + ncAB;
  s.w1Stride = s.w1Tab + tt;
  int t1 = kWarps * s.w1Stride;
  // type 2 fallback: 32-slot table (w, base, vis, U[nE], R[nA], Ka[LBE], Kb[LBE]) + walker state
  s.tab2Stride = (3 + nE + nA + 2 * LBE) | 1;  // odd: conflict-free lane strides
  s.w2Tab = 0;
  s.w2I = 32 * s.tab2Stride;
  s.w2P = s.w2I + kWalkCap;
  s.w2Q = s.w2P + kWalkCap;
  s.w2R = s.w2Q + kWalkCap;
  s.w2Part = s.w2R + kWalkCap;
  s.w2Bits = s.w2Part + kWalkCap;            // kLargeWords uint32
  s.w2Pend = s.w2Bits + kLargeWords / 2;      // 64 int
  s.w2Pref = s.w2Pend + 32;                   // kLargeWords int
  s.w2Stride = s.w2Pref + kLargeWords / 2;
  s.ppMap = kWarps * s.w2Stride;
  s.ppWin = s.ppMap + 2 * maxNP;  // 2 ints per pair
  int t2b = s.ppWin + maxNP;
  int ph = t1;
  if (t2b > ph) ph = t2b;
  s.total = s.phase + ph;
  return s;
}

size_t fast_smem_bytes(int LB, int LE, int cap, int maxNP) {
  return sizeof(double) * (size_t)fast_layout(LB, LE, cap, maxNP).total;
}

struct FastShared {
  // type-2 fallback: break index per primitive pair; during type 1 the
  // primitive pairs ordered by kind (normal, band, zero)
  int ppBreak[kMaxContraction * kMaxContraction];
  int t1Count[3];
  int failIdx[kWalkCap];        // the pass's failed items as (l, l1, l2, l3) bytes
  unsigned failMask[64];
  int nFail, nThis, nextBase;
  int t2Next;                   // next small-grid item to hand out
  unsigned passMask;            // channels read by this pass's failed quadratures
  int passL1, passL2, passL3;   // highest Ka, Kb and r^l rows they read
  int warn;
  unsigned long long estBits;   // mixed path: largest |estimate| of a failed small-grid item (bits)
};

// Mixed path: the largest quadrature value for which double-single level
// sums still decide the large-grid convergence test as FP64 does.  The
// test 16 e^2 <= 3 N |I - q| tol needs the noise of e and I - q, about
// 2^-47 of the integral in double-single, well below 3 N tol / 16; at the
// coarsest levels (N = 256) that noise reaches it for integrals near
// 2^47 tol 48, so quadratures above 1/8 of that take FP64 tables.
__device__ inline double ff_limit(double tol) { return 0x1p47 * tol * 6.0; }

// --------------------------------------------------------------- type 1

// 1/k, k <= 24 (the Legendre recurrence's divisor l - m)
static __device__ const double kRecip[25] = {0.0,        1.0,        1.0 / 2,  1.0 / 3,  1.0 / 4,
                                             1.0 / 5,    1.0 / 6,    1.0 / 7,  1.0 / 8,  1.0 / 9,
                                             1.0 / 10,   1.0 / 11,   1.0 / 12, 1.0 / 13, 1.0 / 14,
                                             1.0 / 15,   1.0 / 16,   1.0 / 17, 1.0 / 18, 1.0 / 19,
                                             1.0 / 20,   1.0 / 21,   1.0 / 22, 1.0 / 23, 1.0 / 24};

// Binomial coefficients C(n, k), n <= 15, as exact doubles: the values
// fac[n] / (fac[n-k] fac[k]) of src/util.c:247-334 (exact integers), looked
// up instead of divided out per term.
struct BinomTable {
  double v[16][16];
  constexpr BinomTable() : v() {
    for (int n = 0; n < 16; n++) {
      v[n][0] = 1.0;
      for (int k = 1; k <= n; k++) v[n][k] = v[n - 1][k - 1] + (k < n ? v[n - 1][k] : 0.0);
    }
  }
};
static __device__ const BinomTable kBinom;
static __device__ inline double binom_tab(int n, int k) { return __ldg(&kBinom.v[n][k]); }

// Direction of the k-vector P as (cos theta, cos phi, sin phi), the values
// src/util.c:75-106 and src/spherical_harmonics.c:16-114 produce through
// theta = acos(z/r), phi = atan(y/x) (+pi) and their cosines and sines,
// computed here without the inverse and direct trigonometric functions (the
// same values within a few ulps; the reference's special cases -- r or x
// below 1e-14 -- are kept).
static __device__ void direction(const double *P, double &ct, double &cp, double &sp) {
  const double eps = 1.0E-14, x = P[0], y = P[1], z = P[2];
  const double r = sqrt(x * x + y * y + z * z);
  ct = r < eps ? 1.0 : fmin(1.0, fmax(-1.0, z / r));
  if (fabs(x) < eps) {
    if (fabs(y) < eps) {
      cp = 1.0;
      sp = 0.0;
    } else {
      const double ph = y < 0.0 ? 1.5 * kPi : 0.5 * kPi;
      cp = cos(ph);
      sp = sin(ph);
    }
  } else {
    const double t = y / x, h = 1.0 / sqrt(1.0 + t * t);  // cos(atan t), sin = t cos
    cp = x > 0.0 ? h : -h;
    sp = x > 0.0 ? t * h : -(t * h);
  }
}

// Column m of the real spherical harmonics S_lm, l = m..lmax, into rsh[l*l +
// l -/+ m]: the associated Legendre recurrence, normalisation and sin/cos(m
// phi) recurrence of src/spherical_harmonics.c:16-114, one column per lane;
// x = cos theta, (c1, s1) = (cos phi, sin phi).
static __device__ void rsh_column(const DevJob &J, int lmax, int m, double x, double c1, double s1,
                                  double *rsh) {
  const int W = J.tmDim + 1;
  double sm = 0.0, cm = 1.0;
  if (m > 0) {
    sm = s1;
    cm = c1;
    for (int i = 2; i <= m; i++) {
      double sn = s1 * cm + c1 * sm, cn = c1 * cm - s1 * sm;
      sm = sn;
      cm = cn;
    }
  }
  double P2 = 0.0, P1 = 0.0, P = 0.0;
  double sp = 1.0;
  if (x != 1.0 && x != -1.0) {
    double st = sqrt(1.0 - x * x);
    sp = st;
    for (int i = 2; i <= m; i++) sp = sp * st;
  }
  for (int l = m; l <= lmax; l++) {
    if (1.0 == x) P = (m == 0) ? 1.0 : 0.0;
    else if (-1.0 == x) P = (m == 0) ? (l == 0 ? 1.0 : -P1) : 0.0;
    else if (l == m) P = (m == 0) ? 1.0 : sp * J.dfac[2 * m - 1];
    else if (l == m + 1) P = x * (2 * m + 1) * P1;
    else P = (x * (2 * l - 1) * P1 - (l + m - 1) * P2) * __ldg(kRecip + (l - m));
    P2 = P1;
    P1 = P;
    double v = J.shNorm[l * W + m] * P;
    if (m == 0) rsh[l * l + l] = v * 0x1.6a09e667f3bcdp-1;  // v / sqrt(2)
    else {
      rsh[l * l + l - m] = v * sm;
      rsh[l * l + l + m] = v * cm;
    }
  }
}

// A group of G primitive pairs (p0 .. p0+G-1) of the type-1 block, by one
// warp (src/type1.c:95-302); lane = (pair, quadrature).  Adds the group's terms
// to the warp's per-combined-index accumulators H.
// The mixed kernel's type-1 large-grid fallback of one primitive pair kk
// (src/type1.c:149-196) for the lanes whose small-grid quadrature (l1, l2)
// failed (`fail`), out of line so that the three pair-kind instances of the
// group code share one copy of both precisions' tables and walks; est: the
// lane's last small-grid estimate (the ff_limit guard).  Returns each failed
// lane's result.
static __device__ __noinline__ double t1_fallback_mixed(const DevJob &J, double *tab, int c, int Lc, int lab, int kk,
                                                       double s, bool fail, double est, int l1, int l2, int Nb,
                                                       const double *pzA, const double *pcA, const double *pzB,
                                                       const double *pcB, double dAC, double dBC, int ws, int we,
                                                       int pa0, int pb0, int &warn) {
  constexpr bool kMixed = true;
  const int lane = threadIdx.x & 31, lq = lab + 1, O = kSmallOrder, OL = J.largeOrder, TSf = 3 + 2 * lq;
  const double *uL = J.uL + (size_t)c * O;
  bool ffp;
  {
    const unsigned hi = (unsigned)((unsigned long long)__double_as_longlong(fail ? est : 0.0) >> 32);
    const unsigned lim = (unsigned)((unsigned long long)__double_as_longlong(ff_limit(J.tol)) >> 32);
    ffp = __reduce_max_sync(0xffffffffu, hi) < lim;
  }
  const double za = pzA[kk / Nb], ca = zeta_times(pcA[kk / Nb], za, pa0), zb = pzB[kk % Nb],
               cb = zeta_times(pcB[kk % Nb], zb, pb0);
  const double z = -za - zb, zd2 = -za * dAC * dAC - zb * dBC * dBC;
  const double C2 = ca * cb;
  const ff C2f = ff_from_double(C2), sf = ff_from_double(s);
  double i1, i2;
  fm06(za, zb, dAC, dBC, i1, i2);
  const ff i1f = ff_from_double(i1);
  // first point past both centres whose exponent is below the screen
  // (src/type1.c:168-176).  Past both centres the exponent falls as r
  // grows, so the predicate is monotone in the index: a 32-way search,
  // first over the last points of 32 chunks, then inside the first chunk
  // whose last point qualifies.
  auto brk = [&](int n) {
    const double r = i1 * J.xLarge[n] + i2, e = (z * r + s) * r + zd2;
    return r > dAC && r > dBC && e < J.lnAcc1;
  };
  const int chunk = (OL + 31) / 32;
  int nb = OL;
  {
    const int n = lane * chunk + chunk - 1 < OL ? lane * chunk + chunk - 1 : OL - 1;
    const unsigned b = __ballot_sync(0xffffffffu, brk(n));
    if (b) {
      const int n0 = (__ffs(b) - 1) * chunk;
      for (int c0 = n0; c0 < n0 + chunk && c0 < OL; c0 += 32) {
        const int m = c0 + lane;
        const unsigned b2 = __ballot_sync(0xffffffffu, m < n0 + chunk && m < OL && brk(m));
        if (b2) {
          nb = c0 + __ffs(b2) - 1;
          break;
        }
      }
    }
  }
  const int end = nb - 1;
  double I2 = 0, p2 = 0, q2 = 0, res2 = 0;
  bool done2 = !fail;
  for (int s0 = 0; s0 < OL;) {
    const int s1 = step_end92(s0) < OL ? step_end92(s0) : OL;
    // the rows the quadratures still running read
    const int kq = __reduce_max_sync(0xffffffffu, done2 ? 0 : l2);
    const int rq = __reduce_max_sync(0xffffffffu, done2 ? 0 : l1);
    for (int t = s0 + lane; t < s1; t += 32) {
      int n = __ldg(J.s92 + t);
      bool upper = t > 0 && ((t - 1) & 1);
      // entry: K_l rows, then the rows w * C2 U_L e^(..) r^l
      double *K = tab + (t - s0) * TSf, *WR = K + lq;
      const double w = J.wLarge[n] * i1;
      bool any = false;
      if (n < nb && !(upper && n > end)) {
        double r = i1 * J.xLarge[n] + i2, ex = (z * r + s) * r + zd2;
        if (ex >= J.lnAcc1) {
          if (ffp) {
            ff *Kf = (ff *)K, *WRf = (ff *)WR;
            const ff rf = ff_from_double(r);
            ff v = ff_mul(ff_mul(J.wLf[n], i1f),
                          ff_mul(C2f, ff_mul(channel_ff(J, c, Lc, rf), ff_exp(ff_from_double(ex)))));
            any = v.hi != 0.0f;
            bessel_ff(J, kq, ff_mul(sf, rf), Kf, 1);
            WRf[0] = v;
            for (int l = 1; l <= rq; l++) {
              v = ff_mul(v, rf);
              WRf[l] = v;
            }
          } else {
            double v = w * (C2 * channel<kMixed>(J, c, Lc, r) * fast_exp(ex));
            any = v != 0.0;
            bessel_fast<kMixed>(J, kq, s * r, K, 1);
            WR[0] = v;
            for (int l = 1; l <= rq; l++) {
              v *= r;
              WR[l] = v;
            }
          }
        }
      } else if (__builtin_expect(n != nb && !upper && n < O && n >= ws && n < we, 0)) {
        // beyond the break the reference integrates its small-grid buffers:
        // exponent and U_L at index n, r^l and K_l at flat offset l*OL + n of
        // rows written with the small grid's stride
        double rs = J.xSmall[n], es = (z * rs + s) * rs;
        if (es >= J.lnAcc1) {
          const double v = w * (C2 * uL[n] * fast_exp(es));
          any = v != 0.0;
          for (int l = 0; l <= lab; l++) {
            int f = l * OL + n, lr = f / O, nr = f % O;
            bool ok = lr <= lab && nr >= ws && nr < we;
            double xr = J.xSmall[nr], pw = 1.0;
            for (int i = 0; i < lr && ok; i++) pw = xr * pw;
            WR[l] = ok ? v * pw : 0.0;
            K[l] = ok ? bessel_row(J, lr, s * xr) : 0.0;
          }
          if (ffp)  // the rows as ff, in place (entry l holds row l either way)
            for (int l = 0; l <= lab; l++) {
              ((ff *)WR)[l] = ff_from_double(WR[l]);
              ((ff *)K)[l] = ff_from_double(K[l]);
            }
        }
      }
      if (!any) {  // zero bits read as 0.0 in FP64 and in ff alike
        for (int l = 0; l <= kq; l++) K[l] = 0.0;
        for (int l = 0; l <= rq; l++) WR[l] = 0.0;
      }
    }
    __syncwarp();
    if (!done2) {
      auto vis = [&](int t) { return c92_slot[t] <= end; };
      if (ffp) {
        auto val = [&](int t) {
          const ff *e = (const ff *)(tab + (t - s0) * TSf);
          return ff_mul(e[lq + l1], e[l2]);
        };
        psm92_advance_ff(s0, s1, J.tol, val, vis, I2, p2, q2, done2, res2);
      } else {
        auto val = [&](int t) {
          const double *e = tab + (t - s0) * TSf;
          return e[lq + l1] * e[l2];
        };
        psm92_advance(s0, s1, J.tol, val, vis, I2, p2, q2, done2, res2);
      }
    }
    __syncwarp();
    s0 = s1;
    if (__all_sync(0xffffffffu, done2)) break;
  }
  double out = 0.0;
  if (fail) {
    if (!done2) {
      res2 = 16 * I2 / (3 * (c92_lvN[c92_nLevels - 1] + 1.0));
      warn = 1;
    }
    out = res2;
  }
  __syncwarp();
  return out;
}

template <bool kMixed, int kKind>
static __device__ void t1_group_run(const DevJob &J, const FastSmem &L, double *W, int c, int Lc,
                                    int la, int lb, const int *perm, int p0, int G, int Nb, const double *pzA,
                                    const double *pcA, const double *pzB, const double *pcB,
                                    const double *gA, const double *gB, int ws, int we, int pa0, int pb0,
                                    int &warn) {
  const int lane = threadIdx.x & 31, lab = la + lb, lq = lab + 1, O = kSmallOrder;
  // odd entry strides: lanes touching neighbouring entries hit distinct banks
  const int OL = J.largeOrder, TSs = 1 + 2 * lq, TSf = 3 + 2 * lq, RQ = lq * lq, nq = t1_items(lab);
  double *sc = W + L.w1Sc, *rsh = W + L.w1Rsh, *Q = W + L.w1Q, *H = W + L.w1H, *tab = W + L.w1Tab;
  const double dAC = gA[3], dBC = gB[3];
  const double *uL = J.uL + (size_t)c * O;
  // (1) per pair: k-vector, its spherical coordinates, the prefactor
  if (lane < G) {
    int k = perm[p0 + lane];
    // derivative blocks: coefficients times zeta^max(0, shift) (src/type1.c:239-246)
    double za = pzA[k / Nb], ca = zeta_times(pcA[k / Nb], za, pa0), zb = pzB[k % Nb],
           cb = zeta_times(pcB[k % Nb], zb, pb0);
    double P[3];
    for (int i = 0; i < 3; i++) P[i] = 2.0 * (za * gA[i] + zb * gB[i]);
    sc[lane * 6 + 0] = sqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);  // |P|, as src/util.c:75-106
    direction(P, sc[lane * 6 + 1], sc[lane * 6 + 2], sc[lane * 6 + 5]);
    sc[lane * 6 + 3] = t1_prefactor(za, ca, zb, cb, dAC, dBC);
    sc[lane * 6 + 4] = -za - zb;
  }
  __syncwarp();
  // (2) S_lm of every pair, one (pair, m) column per lane
  if (lane < G * lq) {
    int g = lane / lq, m = lane % lq;
    rsh_column(J, lab, m, sc[g * 6 + 1], sc[g * 6 + 2], sc[g * 6 + 5], rsh + g * RQ);
  }
  for (int e = lane; e < G * RQ; e += 32) Q[e] = 0.0;
  __syncwarp();
  // (3) small grid, PS93: lane = (pair g, quadrature (l1, l2))
  const bool mine = lane < G * nq;
  const int g = mine ? lane / nq : 0;
  int l1 = 0, l2 = 0;
  {
    int rem = mine ? lane % nq : 0;
    while (l1 <= lab && rem >= l1 / 2 + 1) { rem -= l1 / 2 + 1; l1++; }
    l2 = l1 - 2 * rem;
  }
  double I = 0, p = 0, q = 0;
  bool done = !mine;
  int k = 0, cnt = 0;
  if constexpr (kKind == kPairZero) {
    // converged quadratures add 0 to Q; failed ones go to the fallback
    if (mine) done = t1_zero_walk(J, sc[g * 6], sc[g * 6 + 4], ws, we);
  } else
  for (int s0 = 0; s0 < O;) {
    const int s1 = step_end93(s0) < O ? step_end93(s0) : O;
    // slot entry: [0, lq) K_l(s r), [lq, 2lq) w * C1 U_L e^(..) r^l; zero
    // outside the window.  The step's in-window slots are the run [lo, hi)
    // of its by-point order, dealt to consecutive lanes.
    const int ns = s1 - s0;
    int lo, hi;
    {
      const int n0 = lane < ns ? __ldg(J.s93 + __ldg(J.byN93 + s0 + lane)) : INT_MAX;
      const int n1 = lane + 32 < ns ? __ldg(J.s93 + __ldg(J.byN93 + s0 + lane + 32)) : INT_MAX;
      lo = __popc(__ballot_sync(0xffffffffu, n0 < ws)) + __popc(__ballot_sync(0xffffffffu, n1 < ws));
      hi = __popc(__ballot_sync(0xffffffffu, n0 < we)) + __popc(__ballot_sync(0xffffffffu, n1 < we));
    }
    const int nIn = hi - lo;
    // only the pairs of the group with a quadrature still running are
    // tabulated: a converged lane reads no entry again
    unsigned live = 0;
    {
      const unsigned run = __ballot_sync(0xffffffffu, !done), qm = nq >= 32 ? ~0u : (1u << nq) - 1u;
      for (int gg = 0; gg < G; gg++)
        if (run >> (gg * nq) & qm) live |= 1u << gg;
    }
    const int nLive = __popc(live);
    // the live pairs' indices, 4 bits each (G <= 8), and entry e's (slot,
    // live pair) = (e / nLive, e % nLive) with the quotient by a
    // multiply-shift: ceil(2^16 / d) is exact for d <= 8 and e < 8192
    // (e < 33 * 8 here) -- no integer divide in the loops
    unsigned packed = 0;
    for (unsigned m = live, j = 0; m; m &= m - 1u, j++) packed |= (unsigned)(__ffs(m) - 1) << (4 * j);
    const unsigned dmag = nLive > 0 ? (65536u + (unsigned)nLive - 1u) / (unsigned)nLive : 0u;
    auto slot_of = [&](int e) { return (int)(((unsigned)e * dmag) >> 16); };
    auto live_pair = [&](int e, int i) { return (int)((packed >> (4 * (e - i * nLive))) & 15u); };
    for (int e = lane; e < nIn * nLive; e += 32) {
      const int i = slot_of(e);
      const int gg = live_pair(e, i), t = __ldg(J.byN93 + s0 + lo + i), n = __ldg(J.s93 + t);
      double *ent = tab + ((t - s0) * G + gg) * TSs;
      const double s = sc[gg * 6];
      double *WR = ent + lq;
      if constexpr (kKind == kPairBand) {
        // row l: (C1 r^l) U; the walk multiplies by K, exp(e) and w in turn
        const double r = J.xSmall[n], e = t1_exponent(sc[gg * 6 + 4], s, r), C1 = sc[gg * 6 + 3];
        bessel_fast<kMixed>(J, lab, s * r, ent, 1);
        double R = 1.0;
        for (int l = 0; l <= lab; l++) {
          if (l) R = __dmul_rn(r, R);
          WR[l] = __dmul_rn(__dmul_rn(C1, R), uL[n]);
        }
        ent[2 * lq] = e >= J.lnAcc1 ? fast_exp(e) : 0.0;
      } else {
        double r = J.xSmall[n], ex = (sc[gg * 6 + 4] * r + s) * r;
        ex = ex >= J.lnAcc1 ? fast_exp(ex) : 0.0;
        const double wB = J.wSmall[n] * (sc[gg * 6 + 3] * uL[n] * ex);
        bessel_fast<kMixed>(J, lab, s * r, ent, 1);
        double v = wB;
        WR[0] = v;
        for (int l = 1; l <= lab; l++) {
          v *= r;
          WR[l] = v;
        }
      }
    }
    for (int e = lane; e < (ns - nIn) * nLive; e += 32) {
      const int i = slot_of(e), t = __ldg(J.byN93 + s0 + (i < lo ? i : i + nIn));
      double *ent = tab + ((t - s0) * G + live_pair(e, i)) * TSs;
      for (int l = 0; l <= 2 * lq; l++) ent[l] = 0.0;
    }
    __syncwarp();
    auto ent_of = [&](int t) { return tab + ((t - s0) * G + g) * TSs; };
    // band kind: w * ((((C1 r^l1) U) K_l2) exp(e)), each product rounded
    auto wf = [&](int t, int n) {
      const double *e = ent_of(t);
      return __dmul_rn(J.wSmall[n], __dmul_rn(__dmul_rn(e[lq + l1], e[l2]), e[2 * lq]));
    };
    int t = s0;
    if (t == 0) {
      if (!done) {
        if constexpr (kKind == kPairBand) {
          p = wf(0, c93_slot[0]);
          q = __dadd_rn(wf(1, c93_slot[1]), wf(2, c93_slot[2]));
        } else {
          const double *e0 = ent_of(0), *e1 = ent_of(1), *e2 = ent_of(2);
          p = e0[lq + l1] * e0[l2];
          q = fma(e2[lq + l1], e2[l2], e1[lq + l1] * e1[l2]);
        }
        I = p + q;
      }
      t = 3;
    }
    // the current level's first and end slot, read once per level
    int lvStart = k == 0 ? 3 : c93_lvEnd[k - 1], lvEnd = c93_lvEnd[k];
    while (t < s1) {
      if (t == lvStart) cnt = 0;
      int lo = c93_slot[t], hi = c93_slot[t + 1];
      double T = 0.0;
      if constexpr (kKind == kPairBand) {
        if (lo >= ws) { if (!done) T = wf(t, lo); cnt++; }
        if (hi <= we) { if (!done) T = __dadd_rn(T, wf(t + 1, hi)); cnt++; }
      } else {
        if (lo >= ws) { if (!done) { const double *e = ent_of(t); T = e[lq + l1] * e[l2]; } cnt++; }
        if (hi <= we) { if (!done) { const double *e = ent_of(t + 1); T = fma(e[lq + l1], e[l2], T); } cnt++; }
      }
      if (!done) I += T;
      t += 2;
      if (t == lvEnd) {
        int j = c93_lvJ[k], n = c93_lvN[k];
        if (!done) {
          p += (1 - j) * (I - q);
          // the reference's error estimate is 16 d / (3 n); tested as
          // 16 d < tol 3 n (no divide; the same decision but within an ulp
          // of the threshold)
          const double d = fabs((1 - j) * (q - 3 * p / 2) + j * (I - 2 * q));
          q = (1 - j) * q + j * I;
          if (cnt > 0 && 16 * d < J.tol * (3 * n)) {
            done = true;
            Q[g * RQ + l1 * lq + l2] += 16 * q / (3 * n);
          }
        }
        k++;
        lvStart = lvEnd;
        lvEnd = c93_lvEnd[k];  // k <= the level count, inside the 32-entry table
      }
    }
    __syncwarp();
    s0 = s1;
    if (__all_sync(0xffffffffu, done)) break;
  }
  // (4) large-grid fallback, one pair of the group at a time, for the
  //     quadratures that did not converge (src/type1.c:149-196)
  const bool failed = mine && !done;
  for (int gg = 0; gg < G; gg++) {
    const bool fail = failed && g == gg;
    if (!__ballot_sync(0xffffffffu, fail)) continue;
    // mixed path: the pair's tables in double-single only where the sums of
    // its failed quadratures can take the reference's decisions (ff_limit,
    // judged on their last small-grid estimates); larger integrals in FP64
    if constexpr (kMixed) {
      const double est = fail ? fabs(16 * q / (3 * c93_lvN[c93_nLevels - 1])) : 0.0;
      const double r = t1_fallback_mixed(J, tab, c, Lc, lab, perm[p0 + gg], sc[gg * 6], fail, est, l1, l2, Nb, pzA,
                                         pcA, pzB, pcB, dAC, dBC, ws, we, pa0, pb0, warn);
      if (fail) Q[g * RQ + l1 * lq + l2] += r;
      __syncwarp();
      continue;
    }
    constexpr bool ffp = false;
    const int kk = perm[p0 + gg];
    const double za = pzA[kk / Nb], ca = zeta_times(pcA[kk / Nb], za, pa0), zb = pzB[kk % Nb],
                 cb = zeta_times(pcB[kk % Nb], zb, pb0);
    const double s = sc[gg * 6], z = -za - zb, zd2 = -za * dAC * dAC - zb * dBC * dBC;
    const double C2 = ca * cb;
    const ff C2f = ff_from_double(C2), sf = ff_from_double(s);
    double i1, i2;
    fm06(za, zb, dAC, dBC, i1, i2);
    const ff i1f = ff_from_double(i1);
    // first point past both centres whose exponent is below the screen
    // (src/type1.c:168-176).  Past both centres the exponent falls as r
    // grows, so the predicate is monotone in the index: a 32-way search,
    // first over the last points of 32 chunks, then inside the first chunk
    // whose last point qualifies.
    auto brk = [&](int n) {
      const double r = i1 * J.xLarge[n] + i2, e = (z * r + s) * r + zd2;
      return r > dAC && r > dBC && e < J.lnAcc1;
    };
    const int chunk = (OL + 31) / 32;
    int nb = OL;
    {
      const int n = lane * chunk + chunk - 1 < OL ? lane * chunk + chunk - 1 : OL - 1;
      const unsigned b = __ballot_sync(0xffffffffu, brk(n));
      if (b) {
        const int n0 = (__ffs(b) - 1) * chunk;
        for (int c0 = n0; c0 < n0 + chunk && c0 < OL; c0 += 32) {
          const int m = c0 + lane;
          const unsigned b2 = __ballot_sync(0xffffffffu, m < n0 + chunk && m < OL && brk(m));
          if (b2) {
            nb = c0 + __ffs(b2) - 1;
            break;
          }
        }
      }
    }
    const int end = nb - 1;
    double I2 = 0, p2 = 0, q2 = 0, res2 = 0;
    bool done2 = !fail;
    for (int s0 = 0; s0 < OL;) {
      const int s1 = step_end92(s0) < OL ? step_end92(s0) : OL;
      // the rows the quadratures still running read
      const int kq = __reduce_max_sync(0xffffffffu, done2 ? 0 : l2);
      const int rq = __reduce_max_sync(0xffffffffu, done2 ? 0 : l1);
      for (int t = s0 + lane; t < s1; t += 32) {
        int n = __ldg(J.s92 + t);
        bool upper = t > 0 && ((t - 1) & 1);
        // entry: K_l rows, then the rows w * C2 U_L e^(..) r^l
        double *K = tab + (t - s0) * TSf, *WR = K + lq;
        const double w = J.wLarge[n] * i1;
        bool any = false;
        if (n < nb && !(upper && n > end)) {
          double r = i1 * J.xLarge[n] + i2, ex = (z * r + s) * r + zd2;
          if (ex >= J.lnAcc1) {
            if (ffp) {
              ff *Kf = (ff *)K, *WRf = (ff *)WR;
              const ff rf = ff_from_double(r);
              ff v = ff_mul(ff_mul(J.wLf[n], i1f),
                            ff_mul(C2f, ff_mul(channel_ff(J, c, Lc, rf), ff_exp(ff_from_double(ex)))));
              any = v.hi != 0.0f;
              bessel_ff(J, kq, ff_mul(sf, rf), Kf, 1);
              WRf[0] = v;
              for (int l = 1; l <= rq; l++) {
                v = ff_mul(v, rf);
                WRf[l] = v;
              }
            } else {
              double v = w * (C2 * channel<kMixed>(J, c, Lc, r) * fast_exp(ex));
              any = v != 0.0;
              bessel_fast<kMixed>(J, kq, s * r, K, 1);
              WR[0] = v;
              for (int l = 1; l <= rq; l++) {
                v *= r;
                WR[l] = v;
              }
            }
          }
        } else if (__builtin_expect(n != nb && !upper && n < O && n >= ws && n < we, 0)) {
          // beyond the break the reference integrates its small-grid buffers:
          // exponent and U_L at index n, r^l and K_l at flat offset l*OL + n of
          // rows written with the small grid's stride
          double rs = J.xSmall[n], es = (z * rs + s) * rs;
          if (es >= J.lnAcc1) {
            const double v = w * (C2 * uL[n] * fast_exp(es));
            any = v != 0.0;
            for (int l = 0; l <= lab; l++) {
              int f = l * OL + n, lr = f / O, nr = f % O;
              bool ok = lr <= lab && nr >= ws && nr < we;
              double xr = J.xSmall[nr], pw = 1.0;
              for (int i = 0; i < lr && ok; i++) pw = xr * pw;
              WR[l] = ok ? v * pw : 0.0;
              K[l] = ok ? bessel_row(J, lr, s * xr) : 0.0;
            }
            if (ffp)  // the rows as ff, in place (entry l holds row l either way)
              for (int l = 0; l <= lab; l++) {
                ((ff *)WR)[l] = ff_from_double(WR[l]);
                ((ff *)K)[l] = ff_from_double(K[l]);
              }
          }
        }
        if (!any) {  // zero bits read as 0.0 in FP64 and in ff alike
          for (int l = 0; l <= kq; l++) K[l] = 0.0;
          for (int l = 0; l <= rq; l++) WR[l] = 0.0;
        }
      }
      __syncwarp();
      if (!done2) {
        auto vis = [&](int t) { return c92_slot[t] <= end; };
        if (ffp) {
          auto val = [&](int t) {
            const ff *e = (const ff *)(tab + (t - s0) * TSf);
            return ff_mul(e[lq + l1], e[l2]);
          };
          psm92_advance_ff(s0, s1, J.tol, val, vis, I2, p2, q2, done2, res2);
        } else {
          auto val = [&](int t) {
            const double *e = tab + (t - s0) * TSf;
            return e[lq + l1] * e[l2];
          };
          psm92_advance(s0, s1, J.tol, val, vis, I2, p2, q2, done2, res2);
        }
      }
      __syncwarp();
      s0 = s1;
      if (__all_sync(0xffffffffu, done2)) break;
    }
    if (fail) {
      if (!done2) {
        res2 = 16 * I2 / (3 * (c92_lvN[c92_nLevels - 1] + 1.0));
        warn = 1;
      }
      Q[g * RQ + l1 * lq + l2] += res2;
    }
    __syncwarp();
  }
  __syncwarp();
  // (5) H[p] += sum_l (sum_m S_lm poly2sph[p][lm]) Q[|p|][l], pair by pair in
  //     order (src/type1.c:323-345)
  const int dd = J.tmDim + 1, tmW = (J.tmDim + 1) * (J.tmDim + 1);
  const int ncab = (lab + 1) * (lab + 2) * (lab + 3) / 6;
  for (int pi = lane; pi < ncab; pi += 32) {
    const int *ex = J.ijk + 3 * pi;
    const int lmax = ex[0] + ex[1] + ex[2];
    const int prow = J.ijkIdx[(ex[0] * dd + ex[1]) * dd + ex[2]];
    double acc = H[pi];
    for (int gg = 0; gg < G; gg++) {
      const double *rs = rsh + gg * RQ, *Qg = Q + gg * RQ;
      for (int l = lmax; l >= 0; l -= 2) {
        double factor = 0.0;
        for (int m = 0; m < 2 * l + 1; m++) factor += rs[l * l + m] * J.p2s[(size_t)prow * tmW + l * l + m];
        acc += factor * Qg[lmax * lq + l];
      }
    }
    H[pi] = acc;
  }
  __syncwarp();
}

// --------------------------------------------------------------- type 2

// One primitive pair of the type-2 large-grid fallback, by one warp
// (src/type2.c:418-528): integrates the pass's failed items and adds each
// result to the warp's partial sums.
template <bool kMixed>
static __device__ void t2_pair(const DevJob &J, const FastSmem &L, double *W, const FastShared &S,
                               int k, int Nb, int nf, int c, int Lc, int la, int lb, const double *pzA,
                               const double *pcA, const double *pzB, const double *pcB, double dAC,
                               double dBC, int ncls, int pa0, int pb0, const double *map, const int *win,
                               bool useFF, int &warn) {
  // mixed path: useFF picks the double-single tables and sums for this pass
  // (one copy of the common code for both precisions)
  const bool inFF = kMixed && useFF;
  const int lane = threadIdx.x & 31, nA = 2 * J.maxLBS + 1;
  const int LE = J.maxLECP > 0 ? J.maxLECP : 1, LBE = J.maxLBS + LE, OL = J.largeOrder;
  const int TS = L.tab2Stride;
  double *tab = W + L.w2Tab, *sI = W + L.w2I, *sP = W + L.w2P, *sQ = W + L.w2Q, *sR = W + L.w2R;
  double *part = W + L.w2Part;
  unsigned *needBits = (unsigned *)(W + L.w2Bits);
  int *pend = (int *)(W + L.w2Pend), *pref = (int *)(W + L.w2Pref);
  const double za = pzA[k / Nb], ca = pcA[k / Nb], zb = pzB[k % Nb], cb = pcB[k % Nb];
  // derivative blocks: the product times zeta_a^max(0, shifta), then
  // zeta_b^max(0, shiftb) (src/type2.c:456-462)
  const double Ck = zeta_times(zeta_times(ca * cb, za, pa0), zb, pb0);
  const double i1 = map[2 * k], i2 = map[2 * k + 1];
  const ff i1f = ff_from_double(i1), Ckf = ff_from_double(Ck);
  const int nb = S.ppBreak[k], end = nb == INT_MAX ? OL - 1 : nb - 1;
  const int nLo = win[2 * k], nHi = win[2 * k + 1];
  // the latest break of the earlier pairs: beyond it no earlier pair's
  // buffers are reused
  int mb = -1;
  for (int j = lane; j < k; j += 32) mb = S.ppBreak[j] > mb ? S.ppBreak[j] : mb;
  mb = __reduce_max_sync(0xffffffffu, mb);
  for (int q = lane; q < nf; q += 32) { sI[q] = 0; sP[q] = 0; sQ[q] = 0; sR[q] = 0; }
  for (int w = lane; w < (OL + 31) / 32; w += 32) needBits[w] = 0u;
  __syncwarp();
  // Whose tables slot t reads (the reference's reused buffers): this pair's
  // below its break; beyond it, on the lower half, the last earlier pair
  // whose loop reached that point; and the point, exponent of that pair.
  auto locate = [&](int t, int &owner, double &r, double &ex) {
    const int n = __ldg(J.s92 + t);
    const bool upper = t > 0 && ((t - 1) & 1);
    owner = -1;
    if (n < nb) owner = k;
    else if (__builtin_expect(n != nb && !upper, 0)) {
      for (int j = k - 1; j >= 0; j--)
        if (S.ppBreak[j] >= n) { owner = j; break; }
      if (owner >= 0 && S.ppBreak[owner] == n) owner = -1;
    }
    if (owner < 0) return;
    const double zaj = owner == k ? za : pzA[owner / Nb], zbj = owner == k ? zb : pzB[owner % Nb];
    r = map[2 * owner] * J.xLarge[n] + map[2 * owner + 1];
    const double d1 = dAC - r, d2 = dBC - r;
    ex = -zaj * d1 * d1 - zbj * d2 * d2;
  };
  // A slot needs its tables only where they are not negligible; the others
  // integrate to exactly zero.  Slots are classified step by step (cheap),
  // the needed ones queued, and each pass evaluates 32 queued slots, one per
  // lane, before the quadratures walk every slot up to the first one still
  // queued.
  unsigned doneBits[kWalkCap / 32] = {0u, 0u, 0u, 0u};
  int cpos = 0, wpos = 0, nPend = 0;
  // channels and rows the quadratures still running read (the pass's to
  // begin with, narrowed after every walk)
  unsigned pMask = S.passMask;
  int pL1 = S.passL1, pL2 = S.passL2, pL3 = S.passL3;
  const unsigned below = (1u << lane) - 1u;
  while (wpos < OL) {
    while (nPend < 32 && cpos < OL) {
      const int c1 = step_end92(cpos) < OL ? step_end92(cpos) : OL, t = cpos + lane;
      bool need = false;
      if (t < c1) {
        const int n = __ldg(J.s92 + t);
        if (n < nb) {
          // this pair's own point: only inside its interval can the exponent pass
          if (n >= nLo && n <= nHi) {
            const double r = i1 * J.xLarge[n] + i2, d1 = dAC - r, d2 = dBC - r;
            need = -za * d1 * d1 - zb * d2 * d2 >= J.lnAcc2;
          }
        } else if (n <= mb && n != nb && !(t > 0 && ((t - 1) & 1))) {
          int owner;
          double r, ex;
          locate(t, owner, r, ex);
          need = owner >= 0 && ex >= J.lnAcc2;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, need);
      if (need) {
        pend[nPend + __popc(m & below)] = t;
        atomicOr(&needBits[t >> 5], 1u << (t & 31));
      }
      nPend += __popc(m);
      cpos = c1;
    }
    __syncwarp();
    // this pass: the first queued slots, and the walk's end: an odd slot
    // (whole (lower, upper) pairs) that no queued slot precedes
    int nE = nPend < 32 ? nPend : 32, b = cpos;
    if (nPend > 32) {
      b = pend[32];
      if (!(b & 1)) b -= 1;
      while (nE > 0 && pend[nE - 1] >= b) nE--;
    }
    if (lane < nE) {
      const int t = pend[lane], n = __ldg(J.s92 + t);
      int owner;
      double r, ex;
      locate(t, owner, r, ex);
      // the pair's own exponents (no integer divide) unless a stale slot
      const double zaj = owner == k ? za : pzA[owner / Nb], zbj = owner == k ? zb : pzB[owner % Nb];
      double *e = tab + lane * TS;
      if (inFF) {
        // the same rows in double-single
        ff *U = (ff *)(e + 3), *R = U + LE, *Ka = R + nA, *Kb = Ka + LBE;
        const ff rf = ff_from_double(r);
        const ff wB = ff_mul(ff_mul(J.wLf[n], i1f), ff_mul(Ckf, ff_exp(ff_from_double(ex))));
        channels_ff(J, c, rf, pMask, U);
#pragma unroll 1
        for (int side = 0; side < 2; side++)
          bessel_ff(J, side ? pL2 : pL1, ff_mul(ff_from_double(side ? 2.0 * zbj * dBC : 2.0 * zaj * dAC), rf),
                    side ? Kb : Ka, 1);
        for (int l = 0; l <= pL1; l++) Ka[l] = ff_mul(Ka[l], wB);
        R[0] = {1.0f, 0.0f};
        for (int l = 1; l <= pL3; l++) R[l] = ff_mul(rf, R[l - 1]);
      } else {
        double *U = e + 3, *R = U + LE, *Ka = R + nA, *Kb = Ka + LBE;
        // Ka rows carry the weight and prefactor: w * Ck * e^(..) * K_l1
        const double wB = (J.wLarge[n] * i1) * (Ck * fast_exp(ex));
        // only the channels and rows this pass's quadratures read
        channels_masked<kMixed>(J, c, r, pMask, U);
        // the rows of both centres through one copy of the Bessel code
#pragma unroll 1
        for (int side = 0; side < 2; side++)
          bessel_fast<kMixed>(J, side ? pL2 : pL1, side ? 2.0 * zbj * dBC * r : 2.0 * zaj * dAC * r, side ? Kb : Ka, 1);
        for (int l = 0; l <= pL1; l++) Ka[l] *= wB;
        R[0] = 1.0;
        for (int l = 1; l <= pL3; l++) R[l] = r * R[l - 1];
      }
    }
    if (lane == 0) {  // entry of slot t: queued slots in [wpos, t)
      const int w0 = wpos >> 5, w1 = (b - 1) >> 5;
      int acc = -__popc(needBits[w0] & ((1u << (wpos & 31)) - 1u));
      for (int w = w0; w <= w1; w++) {
        pref[w] = acc;
        acc += __popc(needBits[w]);
      }
    }
    __syncwarp();
    bool all = true;
    unsigned nMask = 0u;
    int n1 = 0, n2 = 0, n3 = 0;
    for (int q = lane, qi = 0; q < nf; q += 32, qi++) {
      if (doneBits[qi] & (1u << lane)) continue;
      // the pass's item, decoded once when the pass was listed
      const int v = S.failIdx[q], l = v & 255, l1 = (v >> 8) & 255, l2 = (v >> 16) & 255, l3 = v >> 24;
      auto entry = [&](int t) {  // a queued slot's table entry
        const unsigned word = needBits[t >> 5], bit = 1u << (t & 31);
        return tab + (pref[t >> 5] + __popc(word & (bit - 1u))) * TS;
      };
      auto vis = [&](int t) { return c92_slot[t] <= end; };  // an upper slot
      double I = sI[q], p = sP[q], qv = sQ[q], res = 0;
      bool done = false;
      if (inFF) {
        auto val = [&](int t) {
          const ff *U = (const ff *)(entry(t) + 3), *R = U + LE, *Ka = R + nA, *Kb = Ka + LBE;
          return ff_mul(ff_mul(ff_mul(Ka[l1], Kb[l2]), U[l]), R[l3]);
        };
        psm92_sparse_ff(wpos, b, needBits, J.tol, val, vis, I, p, qv, done, res);
      } else {
        auto val = [&](int t) {
          const double *e = entry(t);
          const double *U = e + 3, *R = U + LE, *Ka = R + nA, *Kb = Ka + LBE;
          return Ka[l1] * Kb[l2] * U[l] * R[l3];
        };
        psm92_sparse(wpos, b, needBits, J.tol, val, vis, I, p, qv, done, res);
      }
      sI[q] = I; sP[q] = p; sQ[q] = qv;
      if (done) { sR[q] = res; doneBits[qi] |= 1u << lane; }
      else {
        all = false;
        nMask |= 1u << l;
        n1 = l1 > n1 ? l1 : n1;
        n2 = l2 > n2 ? l2 : n2;
        n3 = l3 > n3 ? l3 : n3;
      }
    }
    pMask = __reduce_or_sync(0xffffffffu, nMask);
    pL1 = __reduce_max_sync(0xffffffffu, n1);
    pL2 = __reduce_max_sync(0xffffffffu, n2);
    pL3 = __reduce_max_sync(0xffffffffu, n3);
    // drop the evaluated slots from the queue
    const int rest = nPend - nE;
    const int keep0 = lane < rest ? pend[nE + lane] : 0, keep1 = lane + 32 < rest ? pend[nE + lane + 32] : 0;
    __syncwarp();
    if (lane < rest) pend[lane] = keep0;
    if (lane + 32 < rest) pend[lane + 32] = keep1;
    nPend = rest;
    wpos = b;
    __syncwarp();
    if (__all_sync(0xffffffffu, all)) break;
  }
  const double Nlast = c92_lvN[c92_nLevels - 1] + 1.0;
  for (int q = lane, qi = 0; q < nf; q += 32, qi++) {
    if (doneBits[qi] & (1u << lane)) part[q] += sR[q];
    else { part[q] += 16 * sI[q] / (3 * Nlast); warn = 1; }
  }
  __syncwarp();
}

// --------------------------------------------------------------- the kernel

// One unit (centre c, shell pair pr) by the whole CTA.  Every thread enters
// and leaves together (the early exits are CTA-uniform).
template <bool kMixed>
static __device__ void unit_fast(const DevJob &J, const long long u, FastShared &S, double *sm) {
  const int c = (int)(u / J.nPairs), pr = (int)(u % J.nPairs);
  const int sa = J.pairA[pr], sb = J.pairB[pr], tid = threadIdx.x, NT = blockDim.x;
  const int warp = tid >> 5;
  const int *wa = J.win + ((size_t)c * J.nShells + sa) * 3;
  const int *wb = J.win + ((size_t)c * J.nShells + sb) * 3;
  // derivative shift: the shells' l moved by (shifta, shiftb) for the
  // computation, the blocks handed out with l (lpa, lpb)
  const UnitShift sh = unit_shift(J, pr, J.shL[sa], J.shL[sb], J.shAtom[sa], J.shAtom[sb], J.ctrAtom[c]);
  if (wa[2] || wb[2] || sh.skip) {
    if (tid == 0) J.status[u] = kUnitSkipped;
    return;
  }
  const int ws = wa[0] > wb[0] ? wa[0] : wb[0];
  const int we = wa[1] > wb[1] ? wa[1] : wb[1];
  if (!(ws < we)) {
    if (tid == 0) J.status[u] = kUnitSkipped;
    return;
  }
  const FastSmem Lm = fast_layout(J.maxLBS, J.maxLECP, J.gcap, J.maxNP);
  const int A = J.shAtom[sa], B = J.shAtom[sb], la = J.shL[sa] + sh.a, lb = J.shL[sb] + sh.b, lab = la + lb;
  // the class's type-1 settings (the autotuner may set them per (la, lb))
  const int cls = la * (J.maxLBS + 1) + lb;
  int gcapU = J.gcap, balU = J.balance;
  if (J.classCfg[cls] & kClassSet) {
    gcapU = J.classCfg[cls] & 0xfff;
    balU = (J.classCfg[cls] >> 12) & 1;
  }
  const long long tc0 = J.classCycles ? clock64() : 0;
  const int lpa = sh.lpa, lpb = sh.lpb, pa0 = sh.a > 0 ? sh.a : 0, pb0 = sh.b > 0 ? sh.b : 0;
  const int nA = 2 * J.maxLBS + 1, LE = J.maxLECP > 0 ? J.maxLECP : 1, LBE = J.maxLBS + LE;
  const int Lc = J.ctrL[c], nca = NCUM(la), ncb = NCUM(lb), O = kSmallOrder;
  const size_t cA = (size_t)c * J.nAtoms + A, cB = (size_t)c * J.nAtoms + B;
  const double *gA = J.cgeo + cA * 4, *gB = J.cgeo + cB * 4;
  const double dAC = gA[3], dBC = gB[3];
  const double *pzA = J.primA + J.shP[sa], *pcA = J.primD + J.shP[sa];
  const double *pzB = J.primA + J.shP[sb], *pcB = J.primD + J.shP[sb];
  const int Na = J.shK[sa], Nb = J.shK[sb], NP = Na * Nb;
  double *chi = sm + Lm.chi, *Jsh = sm + Lm.J, *T = sm + Lm.T, *ph = sm + Lm.phase;
  double *out1 = J.out + (size_t)c * J.centreStride + J.pairOff[pr];
  double *out2 = out1 + NCART(lpa) * NCART(lpb);
  int warn1 = 0, warn2 = 0;
  // type-2 small-grid quadratures (src/type2.c:337-387): the items of the
  // unit's class, their F tables (derivative runs max(0, shift),
  // src/type2.c:563-564) and r^k U_l table read through L2
  const int nF = J.nF, nk = J.nk;
  const int nRuns = J.nRuns > 0 ? J.nRuns : 1;
  const double *gFa = J.F + (((size_t)c * J.nShells + sa) * nRuns + pa0) * O * nF;
  const double *gFb = J.F + (((size_t)c * J.nShells + sb) * nRuns + pb0) * O * nF;
  const double *Ut = J.utab + (size_t)c * O * LE * nk;
  const int ncls = (la * (J.maxLBS + 1) + lb) * LE;
  int nItems = 0;
  for (int l = 0; l < Lc; l++) nItems += J.itemCnt[ncls + l];
  auto item = [&](int q, int &l, int &l1, int &l2, int &l3) {
    l = 0;
    while (q >= J.itemCnt[ncls + l]) { q -= J.itemCnt[ncls + l]; l++; }
    int v = J.items[J.itemOff[ncls + l] + q];
    l1 = v & 255; l2 = (v >> 8) & 255; l3 = v >> 16;
  };
  auto tidx = [&](int l, int l1, int l2, int l3) { return ((l * LBE + l1) * LBE + l2) * nA + l3; };
  auto small_item = [&](int q) {
    int l, l1, l2, l3;
    item(q, l, l1, l2, l3);
    double res;
    // FP64 integrand in every mode: the reference's test
    const bool ok = ps93_walk_fast(J.wSmall, ws, we, J.tol,
                                   [&](int n) {
                                     return __ldg(gFa + n * nF + l1) * __ldg(gFb + n * nF + l2) *
                                            __ldg(Ut + ((size_t)n * LE + l) * nk + l3);
                                   },
                                   res);
    if (ok) T[tidx(l, l1, l2, l3)] = res;
    else {
      atomicOr(&S.failMask[q >> 5], 1u << (q & 31));
      atomicAdd(&S.nFail, 1);
      if (kMixed) atomicMax(&S.estBits, (unsigned long long)__double_as_longlong(fabs(res)));
    }
  };
  for (int e = tid; e < LE * LBE * LBE * nA; e += NT) T[e] = 0.0;
  for (int e = tid; e < 64; e += NT) S.failMask[e] = 0;
  if (tid == 0) {
    S.warn = 0;
    S.nFail = 0;
    S.t2Next = 0;
    S.estBits = 0ull;
  }
  __syncthreads();

  // ---------------------------------------------------------- type 1
  {
    double *W = ph + warp * Lm.w1Stride;
    const int ncab = (lab + 1) * (lab + 2) * (lab + 3) / 6;
    for (int e = tid & 31; e < ncab; e += 32) W[Lm.w1H + e] = 0.0;
    __syncwarp();
    // primitive pairs by kind (normal, band, zero), each kind in pair order
    int *perm = S.ppBreak;
    if (warp == 0) {
      const int lane = tid & 31;
      int base[3] = {0, 0, 0};
      for (int k0 = 0; k0 < NP; k0 += 32) {
        const int k = k0 + lane;
        int kind = -1;
        if (k < NP) {
          const double za = pzA[k / Nb], ca = zeta_times(pcA[k / Nb], za, pa0), zb = pzB[k % Nb],
                       cb = zeta_times(pcB[k % Nb], zb, pb0);
          const double C1 = t1_prefactor(za, ca, zb, cb, dAC, dBC);
          double P[3];
          for (int i = 0; i < 3; i++) P[i] = 2.0 * (za * gA[i] + zb * gB[i]);
          const double s2 = P[0] * P[0] + P[1] * P[1] + P[2] * P[2];
          kind = C1 == 0.0 ? kPairZero : (C1 < 0x1p-900 || s2 > 2800.0 * (za + zb)) ? kPairBand : kPairNormal;
        }
        // first pass: counts only
        for (int kd = 0; kd < 3; kd++) base[kd] += __popc(__ballot_sync(0xffffffffu, kind == kd));
      }
      if (lane == 0) { S.t1Count[0] = base[0]; S.t1Count[1] = base[1]; S.t1Count[2] = base[2]; }
      int pos[3] = {0, base[0], base[0] + base[1]};
      for (int k0 = 0; k0 < NP; k0 += 32) {
        const int k = k0 + lane;
        int kind = -1;
        if (k < NP) {
          const double za = pzA[k / Nb], ca = zeta_times(pcA[k / Nb], za, pa0), zb = pzB[k % Nb],
                       cb = zeta_times(pcB[k % Nb], zb, pb0);
          const double C1 = t1_prefactor(za, ca, zb, cb, dAC, dBC);
          double P[3];
          for (int i = 0; i < 3; i++) P[i] = 2.0 * (za * gA[i] + zb * gB[i]);
          const double s2 = P[0] * P[0] + P[1] * P[1] + P[2] * P[2];
          kind = C1 == 0.0 ? kPairZero : (C1 < 0x1p-900 || s2 > 2800.0 * (za + zb)) ? kPairBand : kPairNormal;
        }
        for (int kd = 0; kd < 3; kd++) {
          const unsigned m = __ballot_sync(0xffffffffu, kind == kd);
          if (kind == kd) perm[pos[kd] + __popc(m & ((1u << lane) - 1u))] = k;
          pos[kd] += __popc(m);
        }
      }
    }
    __syncthreads();
    // groups of each kind, dealt to the warps round-robin over all kinds
    int Gk[3], nG[3], nGroups = 0;
    for (int kd = 0; kd < 3; kd++) {
      const int n = S.t1Count[kd];
      int G = t1_group(lab, gcapU);
      // balance: with few primitive pairs, narrower groups keep all warps busy
      if (balU) {
        const int Gb = (n + kWarps - 1) / kWarps;
        if (Gb < G) G = Gb > 0 ? Gb : 1;
      }
      Gk[kd] = G;
      nG[kd] = (n + G - 1) / G;
      nGroups += nG[kd];
    }
    for (int gi = warp; gi < nGroups; gi += kWarps) {
      int kd = 0, gj = gi, off = 0;
      while (gj >= nG[kd]) { gj -= nG[kd]; off += S.t1Count[kd]; kd++; }
      const int p0 = off + gj * Gk[kd], n = S.t1Count[kd] - gj * Gk[kd], G = n < Gk[kd] ? n : Gk[kd];
      if (kd == kPairNormal)
        t1_group_run<kMixed, kPairNormal>(J, Lm, W, c, Lc, la, lb, perm, p0, G, Nb, pzA, pcA, pzB, pcB, gA, gB,
                                          ws, we, pa0, pb0, warn1);
      else if (kd == kPairBand)
        t1_group_run<kMixed, kPairBand>(J, Lm, W, c, Lc, la, lb, perm, p0, G, Nb, pzA, pcA, pzB, pcB, gA, gB,
                                        ws, we, pa0, pb0, warn1);
      else
        t1_group_run<kMixed, kPairZero>(J, Lm, W, c, Lc, la, lb, perm, p0, G, Nb, pzA, pcA, pzB, pcB, gA, gB,
                                        ws, we, pa0, pb0, warn1);
    }
    // the type-2 small-grid quadratures, 32 at a time to whichever warp is
    // through with its type-1 groups (each writes its own entry of T: the
    // result does not depend on the warp)
    for (;;) {
      int q0 = 0;
      if ((tid & 31) == 0) q0 = atomicAdd(&S.t2Next, 32);
      q0 = __shfl_sync(0xffffffffu, q0, 0);
      if (q0 >= nItems) break;
      if (q0 + (tid & 31) < nItems) small_item(q0 + (tid & 31));
    }
    __syncthreads();
    // chi[i][j] = sum over warps of H[index(a_i + b_j)]
    const int dd = J.tmDim + 1;
    for (int e = tid; e < nca * ncb; e += NT) {
      const int *ei = J.ijk + 3 * (e / ncb), *ej = J.ijk + 3 * (e % ncb);
      int pi = J.ijkIdx[((ei[0] + ej[0]) * dd + (ei[1] + ej[1])) * dd + ei[2] + ej[2]];
      double v = 0.0;
      for (int w = 0; w < kWarps; w++) v += ph[w * Lm.w1Stride + Lm.w1H + pi];
      chi[e] = v;
    }
    __syncthreads();
  }
  auto poly_shift = [&](double norm, double *dst) {  // src/util.c:247-334
    const int D = J.uspD, dd = J.tmDim + 1, nta = NCART(lpa), ntb = NCART(lpb);
    const double *uA = J.usp + cA * D * D * D, *uB = J.usp + cB * D * D * D;
    for (int e = tid; e < nta * ncb; e += NT) {
      int c1 = e / ncb, q = e % ncb;
      const int *ex = J.ijk + 3 * (NCUM(lpa - 1) + c1);
      double v = 0.0;
      for (int x = 0; x <= ex[0]; x++) {
        double bx = binom_tab(ex[0], x);
        for (int y = 0; y <= ex[1]; y++) {
          double by = bx * binom_tab(ex[1], y);
          for (int zz = 0; zz <= ex[2]; zz++) {
            double bz = by * binom_tab(ex[2], zz);
            double factor = bz * uA[((ex[0] - x) * D + (ex[1] - y)) * D + (ex[2] - zz)];
            if (fabs(factor) <= J.acc) continue;
            v += factor * chi[J.ijkIdx[(x * dd + y) * dd + zz] * ncb + q];
          }
        }
      }
      Jsh[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < nta * ntb; e += NT) {
      int c1 = e / ntb, c2 = e % ntb;
      const int *ex = J.ijk + 3 * (NCUM(lpb - 1) + c2);
      double v = 0.0;
      for (int x = 0; x <= ex[0]; x++) {
        double bx = binom_tab(ex[0], x);
        for (int y = 0; y <= ex[1]; y++) {
          double by = bx * binom_tab(ex[1], y);
          for (int zz = 0; zz <= ex[2]; zz++) {
            double bz = by * binom_tab(ex[2], zz);
            double factor = bz * uB[((ex[0] - x) * D + (ex[1] - y)) * D + (ex[2] - zz)];
            if (fabs(factor) <= J.acc) continue;
            factor *= norm;
            v += factor * Jsh[c1 * ncb + J.ijkIdx[(x * dd + y) * dd + zz]];
          }
        }
      }
      dst[e] = v;
    }
    __syncthreads();
  };
  const double norm1 = 4.0 * kPi, norm2 = norm1 * norm1;
  poly_shift(norm1, out1);

  // ---------------------------------------------------------- type 2
  // (the small-grid quadratures ran beside the type-1 groups)
  if (S.nFail > 0) {
    // break index of every primitive pair (bisection: the break predicate is
    // monotone in the index beyond both centres)
    double *map = ph + Lm.ppMap;
    int *win = (int *)(ph + Lm.ppWin);
    for (int k = tid; k < NP; k += NT) {
      double za = pzA[k / Nb], zb = pzB[k % Nb], i1, i2;
      fm06(za, zb, dAC, dBC, i1, i2);
      map[2 * k] = i1;
      map[2 * k + 1] = i2;
      int lo = 0, hi = J.largeOrder;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        double r = i1 * J.xLarge[mid] + i2, d1 = dAC - r, d2 = dBC - r;
        double e = -za * d1 * d1 - zb * d2 * d2;
        if (r > dAC && r > dBC && e < J.lnAcc2) hi = mid; else lo = mid + 1;
      }
      S.ppBreak[k] = lo < J.largeOrder ? lo : INT_MAX;
      // point-index interval outside which this pair's exponent stays below
      // the screen by a margin of 1: the exponent is a parabola in r with
      // its vertex at P and r grows with the index
      const double thr = J.lnAcc2 - 1.0, P = (za * dAC + zb * dBC) / (za + zb);
      auto exq = [&](int n) {
        const double r = i1 * J.xLarge[n] + i2, d1 = dAC - r, d2 = dBC - r;
        return -za * d1 * d1 - zb * d2 * d2;
      };
      int a = 0, bb = J.largeOrder;
      while (a < bb) {
        const int mid = (a + bb) >> 1;
        if (i1 * J.xLarge[mid] + i2 >= P) bb = mid; else a = mid + 1;
      }
      const int nv = a;
      a = 0;
      bb = nv;
      while (a < bb) {
        const int mid = (a + bb) >> 1;
        if (exq(mid) >= thr) bb = mid; else a = mid + 1;
      }
      win[2 * k] = a;
      a = nv;
      bb = J.largeOrder;
      while (a < bb) {
        const int mid = (a + bb) >> 1;
        if (exq(mid) < thr) bb = mid; else a = mid + 1;
      }
      win[2 * k + 1] = a - 1;
    }
    if (tid == 0) S.nextBase = 0;
    __syncthreads();
    // passes of up to kWalkCap failed items.  Thread 0 writes the pass's
    // list, count and resume point before the barrier; every thread reads
    // the count after it, and thread 0 writes again only after the pass's
    // last barrier, so no thread can see the next pass's values early.
    for (;;) {
      if (tid == 0) {
        int nf = 0, q = S.nextBase;
        unsigned mask = 0;
        int m1 = 0, m2 = 0, m3 = 0;
        for (; q < nItems && nf < kWalkCap; q++)
          if (S.failMask[q >> 5] & (1u << (q & 31))) {
            int l, l1, l2, l3;
            item(q, l, l1, l2, l3);
            // the item's (l, l1, l2, l3), one byte each (all below 16)
            S.failIdx[nf++] = l | l1 << 8 | l2 << 16 | l3 << 24;
            mask |= 1u << l;
            m1 = l1 > m1 ? l1 : m1;
            m2 = l2 > m2 ? l2 : m2;
            m3 = l3 > m3 ? l3 : m3;
          }
        S.nThis = nf;
        S.nextBase = q;
        S.passMask = mask;
        S.passL1 = m1;
        S.passL2 = m2;
        S.passL3 = m3;
      }
      __syncthreads();
      const int nf = S.nThis;
      if (nf == 0) break;  // no failed item left
      double *W = ph + warp * Lm.w2Stride;
      for (int q = tid & 31; q < nf; q += 32) W[Lm.w2Part + q] = 0.0;
      __syncwarp();
      // mixed path: double-single tables only where their sums can take the
      // reference's decisions (ff_limit); larger integrals in FP64
      const bool ff2 = kMixed && __longlong_as_double((long long)S.estBits) < ff_limit(J.tol);
      for (int k = warp; k < NP; k += kWarps)
        t2_pair<kMixed>(J, Lm, W, S, k, Nb, nf, c, Lc, la, lb, pzA, pcA, pzB, pcB, dAC, dBC, ncls, pa0, pb0,
                        ph + Lm.ppMap, (const int *)(ph + Lm.ppWin), ff2, warn2);
      __syncthreads();
      for (int q = tid; q < nf; q += NT) {
        double v = 0.0;
        for (int w = 0; w < kWarps; w++) v += ph[w * Lm.w2Stride + Lm.w2Part + q];
        const int it = S.failIdx[q];
        T[tidx(it & 255, (it >> 8) & 255, (it >> 16) & 255, it >> 24)] = v;
      }
      __syncthreads();
    }
  }
  // gamma (src/type2.c:583-623)
  {
    const double *angA = J.ang + cA * J.angLam * J.angLM * J.angC;
    const double *angB = J.ang + cB * J.angLam * J.angLM * J.angC;
    const int LMd = J.angLM, AC = J.angC;
    for (int e = tid; e < nca * ncb; e += NT) {
      int pidx = e / ncb, qidx = e % ncb, alpha = 0, beta = 0;
      while (NCUM(alpha) <= pidx) alpha++;
      while (NCUM(beta) <= qidx) beta++;
      double g = 0.0;
      for (int l = 0; l < Lc; l++) {
        int ll1 = l - alpha, p1 = (alpha + l) % 2;
        if (p1 > ll1) ll1 = p1;
        int ll2 = l - beta, p2 = (beta + l) % 2;
        if (p2 > ll2) ll2 = p2;
        double tmp = 0.0;
        for (int l1 = ll1; l1 <= la + l; l1 += 2)
          for (int l2 = ll2; l2 <= lb + l; l2 += 2) {
            double factor = 0.0;
            for (int m = 0; m < 2 * l + 1; m++)
              factor += angA[((size_t)l1 * LMd + l * l + m) * AC + pidx] * angB[((size_t)l2 * LMd + l * l + m) * AC + qidx];
            tmp += factor * T[tidx(l, l1, l2, alpha + beta)];
          }
        g += tmp;
      }
      chi[e] = g;
    }
  }
  __syncthreads();
  poly_shift(norm2, out2);
  if (warn1) atomicOr(&S.warn, 1);
  if (warn2) atomicOr(&S.warn, 2);
  __syncthreads();
  if (tid == 0) {
    int st = (S.warn & 1) ? kUnitWarnType1 : (S.warn & 2) ? kUnitWarnType2 : kUnitDone;
    J.status[u] = st;
    if (st != kUnitDone) atomicMin(&J.errWord[0], (int)u);
    if (J.classCycles) atomicAdd(&J.classCycles[cls], (unsigned long long)(clock64() - tc0));
  }
}

// The screening window and F table of every (shell, centre) -- k_shell_F of
// the drop-in path (src/type2.c:223-310, src/type2.c:149-180) with the
// batched path's Bessel rows and exp; FP64 in every mode.
__global__ void __launch_bounds__(128) k_shell_F_fast(DevJob J) {
  __shared__ int sw[3];
  const int s = blockIdx.x, c = blockIdx.y, O = kSmallOrder;
  const int C = J.ctrAtom[c], A = J.shAtom[s];
  const double *rC = J.geom + 3 * C, *rA = J.geom + 3 * A;
  double x = rC[0] - rA[0], y = rC[1] - rA[1], z = rC[2] - rA[2];
  const double dAC = sqrt(x * x + y * y + z * z);
  if (threadIdx.x == 0) shell_window(J, s, c, dAC, sw);
  __syncthreads();
  // run = derivative order of the table: rows up to L - 1 + l + run and
  // coefficients times zeta^run (src/type2.c:229, :263-290)
  const int nF = J.nF, nRuns = J.nRuns > 0 ? J.nRuns : 1;
  const double *pa = J.primA + J.shP[s], *pd = J.primD + J.shP[s];
  for (int run = 0; run < nRuns; run++) {
    const int lmaxA = J.maxLECP - 1 + J.shL[s] + run;
    double *F = J.F + (((size_t)c * J.nShells + s) * nRuns + run) * O * nF;
    for (int n = threadIdx.x; n < O; n += blockDim.x) {
      double acc[kMaxRows], K[kMaxRows];
      for (int i = 0; i < nF; i++) acc[i] = 0.0;
      if (!sw[2] && n >= sw[0] && n < sw[1] && lmaxA >= 0) {
        double r = J.xSmall[n];
        for (int p = 0; p < J.shK[s]; p++) {
          double zeta = pa[p], da = pd[p];
          for (int k = 0; k < run; k++) da *= zeta;
          bessel_fast<false>(J, lmaxA, 2.0 * zeta * dAC * r, K, 1);
          double e = dAC - r;
          e = fast_exp(-zeta * e * e);
          for (int i = 0; i <= lmaxA; i++) acc[i] += da * K[i] * e;
        }
      }
      for (int i = 0; i < nF; i++) F[(size_t)n * nF + i] = acc[i];
    }
  }
}

// The unit at queue position i (cost order, or the reference's order).
__device__ inline long long queue_unit(const DevJob &J, long long i) { return J.order ? J.order[i] : i; }

// A CTA per unit; blockIdx.x is a queue position.
template <bool kMixed>
__global__ void __launch_bounds__(kUnitThreads, kUnitCtasPerSm) k_unit_fast(DevJob J) {
  extern __shared__ double sm[];
  __shared__ FastShared S;
  const long long i = blockIdx.x;
  unit_fast<kMixed>(J, J.order ? (long long)J.order[i] : i, S, sm);
}

// Persistent CTAs (as many as fit on the GPU) pulling queue positions from
// one counter: the costliest units start first and the cheap ones fill the
// tail, whatever order the hardware would dispatch CTAs in.
template <bool kMixed>
__global__ void __launch_bounds__(kUnitThreads, kUnitCtasPerSm) k_unit_queue(DevJob J) {
  extern __shared__ double sm[];
  __shared__ FastShared S;
  __shared__ long long next;
  // with the screening stage the queue holds the live units only
  const long long n = J.live ? (long long)*J.liveCount : (long long)J.nCentres * J.nPairs;
  // ctaUnits > 0: a CTA takes at most that many units and exits, so that
  // the SMs free up for other launches (the request server's jobs)
  for (int taken = 0; J.ctaUnits <= 0 || taken < J.ctaUnits; taken++) {
    if (threadIdx.x == 0) next = (long long)atomicAdd(J.queueHead, 1ull);
    __syncthreads();
    const long long i = next;
    if (i >= n) break;
    unit_fast<kMixed>(J, J.live ? (long long)J.live[i] : queue_unit(J, i), S, sm);
    __syncthreads();  // shared state is rewritten by the next unit
  }
}

// ---------------------------------------------------------- screening stage

// True when unit u computes blocks: the unit kernels' own early exits (the
// screened windows of src/libecp.c:296-330 and the derivative skip rules).
static __device__ bool unit_live(const DevJob &J, long long u) {
  const int c = (int)(u / J.nPairs), pr = (int)(u % J.nPairs);
  const int sa = J.pairA[pr], sb = J.pairB[pr];
  const int *wa = J.win + ((size_t)c * J.nShells + sa) * 3;
  const int *wb = J.win + ((size_t)c * J.nShells + sb) * 3;
  const UnitShift sh = unit_shift(J, pr, J.shL[sa], J.shL[sb], J.shAtom[sa], J.shAtom[sb], J.ctrAtom[c]);
  if (wa[2] || wb[2] || sh.skip) return false;
  return (wa[0] > wb[0] ? wa[0] : wb[0]) < (wa[1] > wb[1] ? wa[1] : wb[1]);
}

constexpr int kScreenThreads = 256;

// Live units per CTA chunk of the queue.
__global__ void __launch_bounds__(kScreenThreads) k_screen_count(DevJob J, long long n) {
  const long long i = (long long)blockIdx.x * kScreenThreads + threadIdx.x;
  const int live = i < n && unit_live(J, queue_unit(J, i));
  const int cnt = __syncthreads_count(live);
  if (threadIdx.x == 0) J.screenBlocks[blockIdx.x] = cnt;
}

// Exclusive scan of the per-CTA counts (one CTA); the total is the live count.
__global__ void __launch_bounds__(1024) k_screen_scan(DevJob J, int nBlocks) {
  __shared__ int v[1024];
  __shared__ long long base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nBlocks; b0 += 1024) {
    const int b = b0 + threadIdx.x;
    const int x = b < nBlocks ? J.screenBlocks[b] : 0;
    v[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
      const int y = threadIdx.x >= off ? v[threadIdx.x - off] : 0;
      __syncthreads();
      v[threadIdx.x] += y;
      __syncthreads();
    }
    if (b < nBlocks) J.screenBlocks[b] = (int)(base + v[threadIdx.x] - x);
    __syncthreads();
    if (threadIdx.x == 1023) base += v[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *J.liveCount = (unsigned long long)base;
}

// Stable compaction of the live units; the others are marked skipped here.
__global__ void __launch_bounds__(kScreenThreads) k_screen_scatter(DevJob J, long long n) {
  __shared__ int warpCnt[kScreenThreads / 32];
  const long long i = (long long)blockIdx.x * kScreenThreads + threadIdx.x;
  const long long u = i < n ? queue_unit(J, i) : -1;
  const bool live = u >= 0 && unit_live(J, u);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, live);
  if (lane == 0) warpCnt[warp] = __popc(m);
  __syncthreads();
  int pos = J.screenBlocks[blockIdx.x] + __popc(m & ((1u << lane) - 1u));
  for (int w = 0; w < warp; w++) pos += warpCnt[w];
  if (live) J.live[pos] = (int)u;
  else if (u >= 0) J.status[u] = kUnitSkipped;
}

__global__ void k_reset(int *errWord, unsigned long long *queueHead) {
  errWord[0] = INT_MAX;
  errWord[1] = 0;
  if (queueHead) *queueHead = 0ull;
}

// --------------------------------------------------------------- launchers

int upload_schedules_fast(const int *s93slot, int s93n, const int *s93lvEnd, const int *s93lvJ,
                          const int *s93lvN, int s93levels, const int *s92slot, int s92n,
                          const int *s92lvEnd, const int *s92lvN, int s92levels, void *stream) {
  if (s93n > kSmallOrder || s92n > kMaxLargeOrder || s93levels > 32 || s92levels > 32) return 1;
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemcpyToSymbolAsync(c93_slot, s93slot, sizeof(int) * s93n, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c93_lvEnd, s93lvEnd, sizeof(int) * s93levels, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c93_lvJ, s93lvJ, sizeof(int) * s93levels, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c93_lvN, s93lvN, sizeof(int) * s93levels, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c93_nLevels, &s93levels, sizeof(int), 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c92_slot, s92slot, sizeof(int) * s92n, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c92_lvEnd, s92lvEnd, sizeof(int) * s92levels, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c92_lvN, s92lvN, sizeof(int) * s92levels, 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c92_nLevels, &s92levels, sizeof(int), 0, cudaMemcpyHostToDevice, st);
  cudaMemcpyToSymbolAsync(c92_order, &s92n, sizeof(int), 0, cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

void fast_prepare() {
  // function attributes are per device; callers hold the engine lock
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || attr[dev]) return;
  for (const void *k : {(const void *)k_unit_fast<false>, (const void *)k_unit_queue<false>,
                        (const void *)k_unit_fast<true>, (const void *)k_unit_queue<true>}) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    // the whole unified L1/shared array as shared memory: three CTAs of
    // <= 72 KB per SM
    cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  }
  attr[dev] = true;
}

int fast_ctas_per_sm(size_t smemBytes, int queue) {
  fast_prepare();
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, queue ? (const void *)k_unit_queue<false> : (const void *)k_unit_fast<false>,
                                                    kUnitThreads, smemBytes) != cudaSuccess)
    return 0;
  return n;
}

void launch_reset(const DevJob &J, cudaStream_t st) { k_reset<<<1, 1, 0, st>>>(J.errWord, J.queueHead); }

int launch_fast_pipeline(const DevJob &J, cudaStream_t st, size_t smemBytes, const FastConfig &cfg,
                         cudaEvent_t u0, cudaEvent_t u1) {
  fast_prepare();
  if (smemBytes > 200 * 1024) return 3;
  DevJob Jc = J;
  Jc.gcap = cfg.gcap;
  Jc.mixed = cfg.mixed;
  Jc.balance = cfg.balance;
  for (int i = 0; i < kMaxClasses; i++) Jc.classCfg[i] = cfg.cls[i];
  Jc.classCycles = cfg.classCycles;
  if (!cfg.sorted) Jc.order = nullptr;
  else if (cfg.sorted == 2 && J.orderClass) Jc.order = J.orderClass;
  const bool screen = cfg.queue && cfg.screen && J.queueHead && J.live && J.liveCount && J.screenBlocks;
  if (!screen) Jc.live = nullptr;
  launch_prologue(Jc, st, false);
  {
    DevJob Jf = Jc;
    Jf.mixed = 0;  // the F tables stay FP64 in every mode
    k_shell_F_fast<<<dim3(J.nShells, J.nCentres), 128, 0, st>>>(Jf);
  }
  long long nUnits = (long long)J.nCentres * J.nPairs;
  if (screen && nUnits > 0) {  // screening stage: the queue of live units
    const long long nb = (nUnits + kScreenThreads - 1) / kScreenThreads;
    k_screen_count<<<(unsigned)nb, kScreenThreads, 0, st>>>(Jc, nUnits);
    k_screen_scan<<<1, 1024, 0, st>>>(Jc, (int)nb);
    k_screen_scatter<<<(unsigned)nb, kScreenThreads, 0, st>>>(Jc, nUnits);
  }
  if (u0) record_timing(u0, st);
  if (nUnits > 0) {
    if (cfg.queue && J.queueHead) {
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      int per = fast_ctas_per_sm(smemBytes, 1);
      long long grid = (long long)sms * (per > 0 ? per : 1);
      if (J.ctaUnits > 0) {  // bounded CTAs: enough of them for every unit
        const long long need = (nUnits + J.ctaUnits - 1) / J.ctaUnits;
        grid = need > grid ? need : grid;
        if (grid > (1LL << 30)) grid = 1LL << 30;
      }
      if (grid > nUnits) grid = nUnits;
      if (cfg.mixed) k_unit_queue<true><<<(unsigned)grid, kUnitThreads, smemBytes, st>>>(Jc);
      else k_unit_queue<false><<<(unsigned)grid, kUnitThreads, smemBytes, st>>>(Jc);
    } else {
      if (cfg.mixed) k_unit_fast<true><<<(unsigned)nUnits, kUnitThreads, smemBytes, st>>>(Jc);
      else k_unit_fast<false><<<(unsigned)nUnits, kUnitThreads, smemBytes, st>>>(Jc);
    }
  }
  if (u1) record_timing(u1, st);
  launch_epilogue(Jc, st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : kLaunchErrorBase + (int)e;
}

}  // namespace ecpgb

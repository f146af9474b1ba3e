// ecp_device.cuh -- device helpers shared by the kernel translation units.
//
// Included by ecp_fp64.cu (compiled --fmad=false, the drop-in path) and
// ecp_fast.cu (the batched path); each unit gets its own copy of the
// __constant__ level schedules and uploads them itself.
#pragma once
#include <cuda_runtime.h>

#include <climits>
#include <cmath>

#include "ecp_engine.h"
#include "ecp_tables.h"

namespace ecpgb {

#define NCART(l) (((l) + 1) * ((l) + 2) / 2)
#define NCUM(l) (((l) + 1) * ((l) + 2) * ((l) + 3) / 6)

static constexpr double kPi = 3.14159265358979323846;
static constexpr int kMaxRows = 40;   // Bessel rows incl. the 5 Taylor guard rows

static __constant__ int c93_slot[kSmallOrder];
static __constant__ int c93_lvEnd[32], c93_lvJ[32], c93_lvN[32];
static __constant__ int c93_nLevels;
static __constant__ int c92_slot[kMaxLargeOrder];
static __constant__ int c92_lvEnd[32], c92_lvN[32];
static __constant__ int c92_nLevels, c92_order;

// ------------------------------------------------------------ primitives

// K_0..K_lmax(z) = exp(-z) i_l(z) with stride; three branches of
// src/bessel.c:102-199 (small z, 5-term Taylor about the nearest table point,
// asymptotic).  The table is stored transposed: row i holds K_0..K_tabL(z_i).
static __device__ void bessel_eval(const DevJob &J, int lmax, double z, double *K, int stride) {
  if (z < 1.0E-7) {
    if (z <= 0) {
      K[0] = 1.0;
      for (int l = 1; l <= lmax; l++) K[l * stride] = 0.0;
    } else {
      K[0] = 1 - z;
      for (int l = 1; l <= lmax; l++) K[l * stride] = K[(l - 1) * stride] * z / (2 * l + 1);
    }
  } else if (z < 16.0) {
    int top = lmax + 5;
    double d[kMaxRows], prev[kMaxRows];
    double h = J.besselN / 16;  // integer division, as the reference
    int index = (int)floor(z * h + 0.5);
    double dz = z - index / h, scale = 1.0;
    const double *row = J.besT + (size_t)index * (J.tabL + 1);
    for (int l = 0; l <= top; l++) d[l] = row[l];
    for (int l = 0; l <= lmax; l++) K[l * stride] = d[l];
    for (int i = 1; i <= 5; i++) {
      int ti = top - i;
      for (int j = 0; j <= ti + 1; j++) prev[j] = d[j];
      d[0] = prev[1] - prev[0];
      for (int j = 1; j <= ti; j++)
        d[j] = J.besC[j] * (prev[j - 1] - prev[j + 1]) - prev[j] + prev[j + 1];
      scale = scale * dz / i;
      for (int j = 0; j <= lmax; j++) K[j * stride] += scale * d[j];
    }
  } else {
    double A[kMaxRows];
    A[0] = 0.5 / z;
    for (int l = 0; l <= lmax; l++) K[l * stride] = A[0];
    for (int l = 1; l <= lmax; l++) {
      double f = l * (l + 1);
      for (int i = 1; i < l; i++) {
        K[l * stride] += f * A[i];
        f *= (l + i + 1) * (l - i);
      }
      A[l] = -A[0] * A[l - 1] / l;
      K[l * stride] += f * A[l];
    }
  }
}

// Screening window [start, end) of shell s on centre c's small grid and
// whether the shell is screened out entirely (src/type2.c:149-180), written
// to J.win and to w[3]; dAC = |C - A|.  One thread computes it.
static __device__ void shell_window(const DevJob &J, int s, int c, double dAC, int *w) {
  int end = J.gridEnd[c], j;
  double R = J.radius[s], rmin = dAC - R, rmax = dAC + R;
  for (j = end; j >= 0; j--)
    if (J.xSmall[j] < rmin) break;
  w[0] = j + 1;
  for (j = end; j >= 0; j--)
    if (J.xSmall[j] <= rmax) break;
  w[1] = (j < 0 || J.xSmall[j] > rmax) ? -1 : j;
  w[2] = !(w[1] >= w[0]) || R < 0;
  int *g = J.win + ((size_t)c * J.nShells + s) * 3;
  g[0] = w[0]; g[1] = w[1]; g[2] = w[2];
}

// Derivative shifts (src/libecp.c:240-248), indexed [order][shift].
static __constant__ int c_shiftA[3][10] = {{0}, {+1, -1, 0, 0}, {+2, -2, +1, +1, -1, -1, 0, 0, +1, 0}};
static __constant__ int c_shiftB[3][10] = {{0}, {0, 0, +1, -1}, {0, 0, +1, -1, +1, -1, +2, -2, 0, +1}};

// c times z, n times in a row: the reference's zeta^n derivative factors
// (src/type1.c:239-246, src/type2.c:459-462); n <= 0 leaves c.
static __device__ inline double zeta_times(double c, double z, int n) {
  for (int k = 0; k < n; k++) c *= z;
  return c;
}

// The derivative shift of pair entry pr and whether the reference computes
// that (shift, centre) combination at all (src/libecp.c:296-330):
// la, lb are the shells' l; A, B their atoms; C the centre's atom.
struct UnitShift {
  int a, b;       // shifta, shiftb
  int lpa, lpb;   // l of the blocks handed out
  bool skip;
};
static __device__ inline UnitShift unit_shift(const DevJob &J, int pr, int la, int lb, int A, int B, int C) {
  UnitShift s{0, 0, la, lb, false};
  if (!J.pairShift || J.deriv <= 0) return s;
  const int k = J.pairShift[pr], d = J.deriv;
  s.a = c_shiftA[d][k];
  s.b = c_shiftB[d][k];
  s.lpa = la + s.a;
  s.lpb = lb + s.b;
  if (d == 2) {  // src/libecp.c:356-362
    if (s.a == 1 && s.b == 0) s.lpa = la;
    else if (s.a == 0 && s.b == 1) s.lpb = lb;
  }
  s.skip = (A == C && B == C) || la + s.a < 0 || lb + s.b < 0 || (d == 1 && C == A && s.a != 0) ||
           (d == 1 && C == B && s.b != 0);
  return s;
}

// r^n for the ECP exponent n (a double in the interface; integers are the norm).
static __device__ inline double rpow(double r, double n) {
  if (n == 0.0) return 1.0;
  if (n == 1.0) return r;
  if (n == 2.0) return r * r;
  return pow(r, n);
}

// U_l(r) of centre c (src/ecp.c:42-60).
static __device__ double eval_ecp(const DevJob &J, int c, int l, double r) {
  double pot = 0.0, r2 = r * r;
  int t0 = J.ctrT0[c], t1 = t0 + J.ctrNT[c];
  for (int t = t0; t < t1; t++)
    if (J.termL[t] == l) pot += rpow(r, J.termN[t]) * J.termD[t] * exp(-J.termA[t] * r2);
  return pot;
}

// (r, theta, phi); src/util.c:75-106.
static __device__ void to_spherical(const double *v, double *out) {
  const double eps = 1.0E-14;
  double x = v[0], y = v[1], z = v[2];
  double r = sqrt(x * x + y * y + z * z), th, ph;
  th = (r < eps) ? 0.0 : acos(z / r);
  if (fabs(x) < eps) {
    if (fabs(y) < eps) ph = 0.0;
    else if (y < 0.0) ph = 1.5 * kPi;
    else ph = 0.5 * kPi;
  } else {
    ph = (x > 0.0) ? atan(y / x) : atan(y / x) + kPi;
  }
  out[0] = r; out[1] = th; out[2] = ph;
}

// Real spherical harmonics, index l*l + l + m (m = -l..l);
// src/spherical_harmonics.c:16-114.  lmax <= 12.
static __device__ void real_sph(const DevJob &J, int lmax, double theta, double phi, double *rsh) {
  double P[169], s[14], c[14];
  int n = (lmax + 1) * (lmax + 1);
  for (int i = 0; i < n; i++) P[i] = 0.0;
  for (int i = 0; i < 14; i++) { s[i] = 0.0; c[i] = 0.0; }
#define PL(l, m) P[(l) * (l) + (m) + (l)]
  double x = cos(theta);
  if (1.0 == x) {
    for (int l = 0; l <= lmax; l++) PL(l, 0) = 1.0;
  } else if (-1.0 == x) {
    PL(0, 0) = 1.0;
    for (int l = 1; l <= lmax; l++) PL(l, 0) = -PL(l - 1, 0);
  } else {
    s[1] = sqrt(1.0 - x * x);
    for (int l = 2; l <= lmax; l++) s[l] = s[l - 1] * s[1];
    for (int l = 0; l <= lmax; l++) {
      if (l == 0) { PL(0, 0) = 1.0; continue; }
      PL(l, l) = s[l] * J.dfac[2 * l - 1];
      int m = l - 1;
      PL(l, m) = x * (2 * m + 1) * PL(l - 1, m);
      if (l > 1)
        for (m = 0; m <= l - 2; m++)
          PL(l, m) = (x * (2 * l - 1) * PL(l - 1, m) - (l + m - 1) * PL(l - 2, m)) / (l - m);
    }
  }
  for (int l = 0; l <= lmax; l++) {
    double norm0 = sqrt((2.0 * l + 1.0) / (2.0 * kPi));
    PL(l, 0) = norm0 * PL(l, 0);
    for (int m = 1; m <= l; m++) {
      double norm = sqrt(J.fac[l - m] / J.fac[l + m]) * norm0;
      PL(l, m) = norm * PL(l, m);
    }
  }
  if (lmax > 0) {
    if (0.0 == phi) {
      for (int m = 0; m <= lmax; m++) { s[m] = 0.0; c[m] = 1.0; }
    } else {
      s[1] = sin(phi);
      c[1] = cos(phi);
      for (int m = 2; m <= lmax; m++) {
        s[m] = s[1] * c[m - 1] + c[1] * s[m - 1];
        c[m] = c[1] * c[m - 1] - s[1] * s[m - 1];
      }
    }
  }
  for (int l = 0; l <= lmax; l++) {
    rsh[l * l + l] = PL(l, 0) / sqrt(2.0);
    for (int m = 1; m <= l; m++) {
      rsh[l * l + l - m] = PL(l, m) * s[m];
      rsh[l * l + l + m] = PL(l, m) * c[m];
    }
  }
#undef PL
}

// Squared radius where c r^l exp(-zeta r^2) = cutoff; -1 if Newton fails
// (src/util.c:134-172, where the reference asserts).
static __device__ double gto_radius(double c, double zeta, int l, double cutoff) {
  double delta, dg, guess, zr, r;
  const double t = log(fabs(c) / fabs(cutoff));
  dg = t / zeta;
  r = (dg > cutoff) ? dg : cutoff;
  if (l != 0) {
    bool ok = false;
    if (l > 0) {
      dg = sqrt(0.5 * l / fabs(c));
      guess = (dg > cutoff) ? dg : cutoff;
      if (guess > r) r = 0.5 * (r + guess);
    }
    for (int i = 0; i < 40; i++) {
      zr = zeta * r;
      guess = t + l * log(r) - zr * r;
      delta = guess / (l / r - 2 * zr);
      dg = r - delta;
      r = (dg > cutoff) ? dg : cutoff;
      if (fabs(delta) < cutoff) { r *= r; ok = true; break; }
    }
    if (!ok) return -1.0;
  }
  return r;
}

static __device__ inline double binom(const double *fac, int n, int k) {
  return (k >= 0 && k <= n) ? fac[n] / (fac[n - k] * fac[k]) : 0.0;
}

// ------------------------------------------------------------ quadratures

// Adaptive PS93 walk over the small grid (src/gc_integrators.c:157-217):
// `f(n)` is the integrand at abscissa index n; lower-half points count from
// `start`, upper-half points up to `end`; a level that touches no point skips
// the absolute error test.
// rel > 0 (the batched mixed mode only) also accepts a level of at least 63
// points whose error estimate is below rel times the estimate itself; rel = 0
// is the reference's test exactly (the error estimate is never negative).
template <class Fn>
static __device__ bool ps93_walk(const double *w, int start, int end, double tol, double rel, Fn f,
                                 double &res) {
  int mid = c93_slot[0], a = c93_slot[1], b = c93_slot[2];
  double p = w[mid] * f(mid);
  double q = w[a] * f(a) + w[b] * f(b);
  double I = p + q, err = 0.0;
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
    if (cnt > 0) err = 16 * fabs((1 - j) * (q - 3 * p / 2) + j * (I - 2 * q)) / (3 * n);
    q = (1 - j) * q + j * I;
    if (cnt == 0) continue;
    if (err < tol || (n >= 63 && err < rel * fabs(16 * q / (3 * n)))) {
      res = 16 * q / (3 * n);
      return true;
    }
  }
  return false;
}

// PSM92 walk state (src/gc_integrators.c:39-86) advanced chunk by chunk over
// the schedule.  st = {I, p, q, result}; done = 1 converged.
struct Walk {
  double *I, *p, *q, *res;
  int *done;
};

// Level of schedule slot pos (pos >= 1).
static __device__ inline int level_of(int pos) {
  int k = 0;
  while (c92_lvEnd[k] <= pos) k++;
  return k;
}

}  // namespace ecpgb

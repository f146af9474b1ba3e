// ecp_tables.cpp -- init-time tables of the ECP engine (host side, FP64).
//
// Each builder states the reference code whose table it reproduces; the
// arithmetic is kept in the same operation order so that the device sees the
// same table values the reference computes.
#include "ecp_tables.h"

#include <cmath>
#include <cstdlib>

namespace ecpgb {
void split_pairs(const std::vector<double> &d, std::vector<float> &out);

static const double kPi = 3.14159265358979323846;

// n! / n!! up to `top`; src/util.c:57-100 (f[0] = f[1] = 1, f[i] = f[i-step]*i).
static bool fact_table(int top, int step, std::vector<double> &f) {
  f.assign(top + 1, 0.0);
  f[0] = 1.0;
  if (top >= 1) f[1] = 1.0;
  for (int i = 2; i <= top; i++) {
    f[i] = f[i - step] * i;
    if (std::isinf(f[i])) return false;
  }
  return true;
}

static double binom(int n, int k, const std::vector<double> &fac) {
  return (k >= 0 && k <= n) ? fac[n] / (fac[n - k] * fac[k]) : 0.0;
}

static int tm_dim(int l, const std::vector<double> &fac) {  // src/transformations.h:13
  return (int)((3 * l + 2) * fac[l + 3] / (12 * fac[l]));
}

// Cartesian exponents, libint order; src/dimensions.c:18-58.
static void cart_tables(int am, std::vector<int> &ijk, std::vector<int> &index) {
  ijk.assign(3 * ncum(am), 0);
  int d = am + 1;
  index.assign(d * d * d, 0);
  for (int l = 0; l <= am; l++) {
    int c = 0;
    for (int i = 0; i <= l; i++)
      for (int j = 0; j <= i; j++, c++) {
        int k = ncum(l - 1) + c;
        ijk[3 * k] = l - i;
        ijk[3 * k + 1] = i - j;
        ijk[3 * k + 2] = j;
        index[((l - i) * d + (i - j)) * d + j] = k;
      }
  }
}

// Cartesian -> real spherical (Schlegel & Frisch 1995, eq. 15), blocks
// [l][m][c]; src/transformations.c:29-87.
static void cart2sph(int lmax, const std::vector<int> &xyz, const std::vector<double> &fac,
                     std::vector<double> &TM) {
  TM.assign(tm_dim(lmax, fac), 0.0);
  size_t t = 0;
  for (int l = 0; l <= lmax; l++)
    for (int m = -l; m <= l; m++) {
      int mm = std::abs(m);
      for (int c = 0; c < ncart(l); c++, t++) {
        const int *e = &xyz[3 * (ncum(l - 1) + c)];
        int lx = e[0], ly = e[1], lz = e[2];
        int j = lx + ly - mm;
        if (j < 0 || j % 2 == 1) { TM[t] = 0.0; continue; }
        j /= 2;
        double s1 = 0.0;
        for (int i = 0; i <= (l - mm) / 2; i++) {
          double s2 = 0.0;
          for (int k = 0; k <= j; k++) {
            double s = 0.0;
            if ((m < 0 && std::abs(mm - lx) % 2 == 1) || (m > 0 && std::abs(mm - lx) % 2 == 0))
              s = std::pow(-1.0, (mm - lx + 2 * k) / 2) * std::sqrt(2.0);
            else if (m == 0 && lx % 2 == 0)
              s = std::pow(-1.0, -lx / 2 + k);
            s2 += binom(j, k, fac) * binom(mm, lx - 2 * k, fac) * s;
          }
          s1 += binom(l, i, fac) * binom(i, j, fac) * std::pow(-1.0, i) * fac[2 * l - 2 * i] /
                fac[l - mm - 2 * i] * s2;
        }
        TM[t] = std::sqrt((fac[2 * lx] * fac[2 * ly] * fac[2 * lz] * fac[l] * fac[l - mm]) /
                          (fac[2 * l] * fac[lx] * fac[ly] * fac[lz] * fac[l + mm])) *
                1 / (std::pow(2.0, l) * fac[l]) * s1;
      }
    }
}

// Unit-sphere polynomial -> real spherical harmonic expansion
// (Flores-Moreno et al. 2006, eq. 36); src/transformations.c:147-207.
static void poly2sph(const std::vector<double> &M, int lmax, const std::vector<int> &xyz,
                     const std::vector<double> &dfac, std::vector<double> &TM) {
  int ldim = nsph(lmax);
  TM.assign((size_t)ncum(lmax) * ldim, 0.0);
  for (int l1 = 0; l1 <= lmax; l1++)
    for (int c1 = 0; c1 < ncart(l1); c1++) {
      const int *e1 = &xyz[3 * (ncum(l1 - 1) + c1)];
      double *T = &TM[(size_t)(ncum(l1 - 1) + c1) * ldim];
      size_t tcs = 0;
      for (int l2 = 0; l2 <= l1; l2++) {
        double s1 = 4.0 * kPi * dfac[2 * l2 + 1];
        for (int m = 0; m < 2 * l2 + 1; m++) {
          double sum = 0.0;
          for (int c2 = 0; c2 < ncart(l2); c2++, tcs++) {
            const int *e2 = &xyz[3 * (ncum(l2 - 1) + c2)];
            int lx = e1[0] + e2[0], ly = e1[1] + e2[1], lz = e1[2] + e2[2];
            if (lx % 2 || ly % 2 || lz % 2) continue;
            double s = s1, s2 = 1.0 / dfac[l1 + l2 + 1];
            if (lx > 2) s2 *= dfac[lx - 1];
            if (ly > 2) s2 *= dfac[ly - 1];
            if (lz > 2) s2 *= dfac[lz - 1];
            if (e2[0] > 1) s /= dfac[2 * e2[0] - 1];
            if (e2[1] > 1) s /= dfac[2 * e2[1] - 1];
            if (e2[2] > 1) s /= dfac[2 * e2[2] - 1];
            sum += std::sqrt(s) * s2 * M[tcs];
          }
          *T++ = sum;
        }
      }
    }
}

// --------------------------------------------------------------- grids

// PS93 schedule: simulates the index arithmetic of integrateGC_PS93
// (src/gc_integrators.c:157-217) once, so the kernels walk a table.
static void schedule_ps93(int nParam, Schedule &s) {
  int runs = (int)std::floor(std::log(nParam) / std::log(2));
  int offset = (int)std::pow(2, runs);
  int order = 3 * offset - 1;
  int n = 3, j = 0;
  s = Schedule();
  s.order = order;
  s.headCount = 3;
  s.slot = {(order - 1) / 2, offset - 1, order - offset};
  offset /= 2;
  while ((2 * n * (1 - j) + j * 4 * n / 3 - 1) <= order) {
    j = 1 - j;
    if (j == 0) offset /= 2;
    for (int i = 1; i < n; i += 2)
      if (3 * ((i + 2 * j) / 3) >= i + j) {
        int lo = i * offset - 1;
        s.slot.push_back(lo);
        s.slot.push_back(order - lo - 1);
      }
    n *= (1 + j);
    s.lvEnd.push_back((int)s.slot.size());
    s.lvJ.push_back(j);
    s.lvN.push_back(n);
  }
  s.nLevels = (int)s.lvEnd.size();
}

// PSM92 schedule (src/gc_integrators.c:39-86).
static void schedule_psm92(int gridOrder, Schedule &s) {
  int order = (int)std::pow(2, std::floor(std::log(gridOrder + 1) / std::log(2))) - 1;
  int runs = (int)std::floor(std::log(order) / std::log(2));
  int offset = (int)std::pow(2, runs);
  int M = (order - 1) / 2, n = 1;
  s = Schedule();
  s.order = order;
  s.headCount = 1;
  s.slot = {M};
  while (n <= M) {
    offset /= 2;
    for (int i = 1; i <= n; i += 2) {
      int lo = i * offset - 1;
      s.slot.push_back(lo);
      s.slot.push_back(order - lo - 1);
    }
    n = 2 * n + 1;
    s.lvEnd.push_back((int)s.slot.size());
    s.lvJ.push_back(0);
    s.lvN.push_back(n);
  }
  s.nLevels = (int)s.lvEnd.size();
}

// PS93 abscissae and weights, then the Krack-Koster map (0, inf);
// src/gc_integrators.c:221-283 and :302-315.
static void grid_ps93(int maxPoints, std::vector<double> &x, std::vector<double> &w) {
  int runs = (int)std::floor(std::log(maxPoints) / std::log(2));
  int offset = (int)std::pow(2, runs);
  int order = 3 * offset - 1, n = 3;
  double C0 = std::sin(kPi / 3), S0 = 0.5, C1 = S0, S1 = C0, c, s, s2, t;
  x.assign(order, 0.0);
  w.assign(order, 0.0);
  c = std::cos(kPi / 3);
  s = C0;
  s2 = s * s;
  x[order / 2] = 0.0;
  w[order / 2] = 1.0;
  t = (n - 2.0) / n + 2 / kPi * (1 + 2 * s2 / 3) * c * s;
  x[offset - 1] = -t;
  x[order - offset] = t;
  w[order - offset] = w[offset - 1] = s2 * s2;
  while ((4 * n / 3 - 1) <= order) {
    c = C0;
    s = S0;
    offset /= 2;
    for (int i = 1; i < n; i += 2) {
      int idx = i * offset - 1;
      s2 = s * s;
      t = 1 + 2 / (3 * kPi) * s * c * (3 + 2 * s2) - ((double)i) / n;
      x[idx] = -t;
      x[order - idx - 1] = t;
      w[order - idx - 1] = w[idx] = s2 * s2;
      t = s;
      s = s * C1 + c * S1;
      c = c * C1 - t * S1;
    }
    n *= 2;
    C1 = C0;
    S1 = S0;
    C0 = std::sqrt((1 + C0) / 2);
    S0 = S0 / (2 * C0);
  }
  double ln2 = std::log(2.0);
  for (int i = 0; i < order; i++) {
    double xi = 1.0 - std::log(1.0 - x[i]) / ln2;
    double wi = w[i] / (ln2 * (1.0 - x[i]));
    x[i] = xi;
    w[i] = wi;
  }
}

// PSM92 abscissae and weights on (-1, 1); src/gc_integrators.c:90-145.
static void grid_psm92(int maxPoints, std::vector<double> &x, std::vector<double> &w) {
  int order = (int)std::pow(2, std::floor(std::log(maxPoints + 1) / std::log(2))) - 1;
  int runs = (int)std::floor(std::log(order) / std::log(2));
  int offset = (int)std::pow(2, runs);
  int M = (order - 1) / 2, n = 1;
  double N = n + 1.0, S0 = 1.0, C0 = 0.0, S1, C1, s, c, t;
  x.assign(order, 0.0);
  w.assign(order, 0.0);
  x[M] = 0.0;
  w[M] = 1.0;
  while (n <= M) {
    C1 = C0;
    S1 = S0;
    C0 = std::sqrt((1 + C1) / 2);
    S0 = S1 / (2 * C0);
    s = S0;
    c = C0;
    offset /= 2;
    for (int i = 1; i <= n; i += 2) {
      t = 1 + 2 / (3 * kPi) * (3 + 2 * s * s) * s * c - i / N;
      int idx = i * offset - 1;
      x[order - idx - 1] = t;
      x[idx] = -t;
      w[order - idx - 1] = w[idx] = s * s * s * s;
      t = s;
      s = s * C1 + c * S1;
      c = c * C1 - t * S1;
    }
    n = 2 * n + 1;
    N = n + 1.0;
  }
}

// Series table of K_l(z) = exp(-z) i_l(z) at z = i/(N/16), i = 0..N
// (Flores-Moreno et al. 2006, App. B); src/bessel.c:20-82.  Stored
// transposed, [i][l], so one evaluation reads one contiguous row.
static bool bessel_table(int lMax, int N, int cutoff, double accuracy, std::vector<double> &KT,
                         std::vector<double> &Cc) {
  int dim = N + 1, W = lMax + 1;
  std::vector<double> K((size_t)W * dim, 0.0), F(cutoff + 1), G(cutoff + lMax + 2);
  K[0] = 1.0;
  for (int i = 1; i <= N; i++) {
    double z = i / (N / 16.0), f = z * z / 2.0, s;
    int j = 0, l;
    F[0] = std::exp(-z);
    G[0] = 1.0;
    s = F[0] / G[0];
    l = (int)(0.25 * std::sqrt(1.0 + 16.0 * f));
    while (s > accuracy || j <= l) {
      K[i] += s;
      j++;
      if (j > cutoff) return false;
      F[j] = F[j - 1] * f / j;
      G[j] = G[j - 1] * (2.0 * j + 1.0);
      s = F[j] / G[j];
    }
    for (l = 1; l <= lMax; l++) G[j + l] = G[j + l - 1] * (2 * j + 2 * l + 1);
    f = z;
    for (l = 1; l <= lMax; l++) {
      s = 0;
      for (int m = 0; m < j; m++) s += F[m] / G[l + m];
      K[(size_t)l * dim + i] = f * s;
      f *= z;
    }
  }
  KT.assign((size_t)dim * W, 0.0);
  for (int l = 0; l < W; l++)
    for (int i = 0; i < dim; i++) KT[(size_t)i * W + l] = K[(size_t)l * dim + i];
  Cc.assign(W, 0.0);
  for (int i = 1; i <= lMax; i++) Cc[i] = i / (2.0 * i + 1.0);
  return true;
}

// Angular table Omega[lm][lambda mu][Cartesian alpha] (basis- and
// ECP-independent); src/angular_integrals.c:16-101.
static void omega_table(HostTables &t) {
  int maxL = t.maxLECP, tmW = nsph(t.tmDim), d = t.tmDim + 1;
  t.omD1 = nsph(t.maxLambda);
  t.omD2 = ncum(t.maxAlpha);
  int inc1 = t.omD2, inc2 = t.omD1 * t.omD2;
  t.omega.assign((size_t)nsph(maxL) * inc2 + 1, 0.0);
  for (int lam = 0; lam <= t.maxLambda; lam++)
    for (int l = 0; l < maxL; l++) {
      int par = (lam + l) % 2, lo = lam - l;
      int minAlpha = par > lo ? par : lo;
      for (int alpha = minAlpha; alpha <= t.maxAlpha; alpha += 2)
        for (int mu = 0; mu < 2 * lam + 1; mu++)
          for (int m = 0; m < 2 * l + 1; m++) {
            double *cijk = &t.omega[(size_t)(l * l + m) * inc2 + (lam * lam + mu) * inc1 + ncum(alpha - 1)];
            for (int c = 0; c < ncart(alpha); c++) {
              const int *e = &t.ijk[3 * (ncum(alpha - 1) + c)];
              if (alpha == 0) {
                if (l == lam && m == mu) cijk[c] = 1.0;
              } else if (lam <= l + alpha) {
                for (int dd = 0; dd < ncart(l); dd++) {
                  const int *f = &t.ijk[3 * (ncum(l - 1) + dd)];
                  double N = 0.25 * t.dfac[2 * l + 1] / kPi;
                  if (f[0] > 1) N /= t.dfac[2 * f[0] - 1];
                  if (f[1] > 1) N /= t.dfac[2 * f[1] - 1];
                  if (f[2] > 1) N /= t.dfac[2 * f[2] - 1];
                  N = std::sqrt(N);
                  int p = t.ijkIndex[((f[0] + e[0]) * d + (f[1] + e[1])) * d + (f[2] + e[2])];
                  int ti = l == 0 ? 0 : tm_dim(l - 1, t.fac) + m * ncart(l) + dd;
                  cijk[c] += N * t.cart2sph[ti] * t.poly2sph[(size_t)p * tmW + lam * lam + mu];
                }
              }
            }
          }
    }
}

void build_tables(const TableKey &key, HostTables &t) {
  t = HostTables();
  t.key = key;
  t.maxLECP = key.maxLECP;
  t.maxLBS = key.maxLBS;
  t.maxAlpha = key.maxLBS;
  t.maxLambda = key.maxLECP - 1 + t.maxAlpha;
  if (key.maxLBS < 0 || key.maxLBS > kMaxLBasis || key.maxLECP < 0 || key.maxLECP > kMaxLEcp ||
      key.largeGridOrder < 384 || key.largeGridOrder > 1 << 16) {
    t.status = 3;
    return;
  }
  // The reference sizes these by maxLambda + maxAlpha; rows beyond that are
  // read by pairs with la + lb > maxLambda (out of bounds there).  Values of
  // every in-bounds entry do not depend on the sizes.
  t.tmDim = t.maxLambda + t.maxAlpha;
  if (t.tmDim < 2 * t.maxLBS) t.tmDim = 2 * t.maxLBS;
  if (t.tmDim < 1) t.tmDim = 1;
  if (t.maxLambda < 0) t.maxLambda = 0;
  t.nk = (t.maxLambda > 2 * t.maxLBS ? t.maxLambda : 2 * t.maxLBS) + 1;
  t.nF = t.maxLECP - 1 + t.maxLBS + 1;
  if (t.nF < 1) t.nF = 1;
  if (!fact_table(2 * t.tmDim + 4, 1, t.fac) || !fact_table(2 * t.tmDim + 4, 2, t.dfac)) {
    t.status = 3;
    return;
  }
  cart_tables(t.tmDim, t.ijk, t.ijkIndex);
  if (!key.ordering.empty()) {  // the caller's order within each shell (src/libecp.c:159-165)
    if (key.ordering.size() < t.ijk.size()) {
      t.status = 3;
      return;
    }
    const int d = t.tmDim + 1;
    for (size_t k = 0; k < t.ijk.size() / 3; k++) {
      for (int c = 0; c < 3; c++) t.ijk[3 * k + c] = key.ordering[3 * k + c];
      t.ijkIndex[(t.ijk[3 * k] * d + t.ijk[3 * k + 1]) * d + t.ijk[3 * k + 2]] = (int)k;
    }
  }
  cart2sph(t.tmDim, t.ijk, t.fac, t.cart2sph);
  poly2sph(t.cart2sph, t.tmDim, t.ijk, t.dfac, t.poly2sph);
  grid_ps93(128, t.xs, t.ws);
  schedule_ps93(128, t.s93);
  grid_psm92(key.largeGridOrder, t.xl, t.wl);
  split_pairs(t.xl, t.xlf);
  split_pairs(t.wl, t.wlf);
  schedule_psm92((int)t.xl.size(), t.s92);
  t.tabL = t.maxLECP + t.maxAlpha + 6;
  if (t.tabL < 2 * t.maxLBS + 5) t.tabL = 2 * t.maxLBS + 5;
  if (!bessel_table(t.tabL, t.besselN, 200, key.accuracy, t.besselT, t.besselC)) {
    t.status = 1;
    return;
  }
  if (t.maxLECP > 0) omega_table(t);
  else t.omega.assign(1, 0.0);
  bessel_horner(t);
  const int W = t.tmDim + 1;
  t.shNorm.assign((size_t)W * W, 0.0);
  for (int l = 0; l < W; l++) {
    double norm0 = std::sqrt((2.0 * l + 1.0) / (2.0 * kPi));
    t.shNorm[(size_t)l * W] = norm0;
    for (int m = 1; m <= l; m++) t.shNorm[(size_t)l * W + m] = std::sqrt(t.fac[l - m] / t.fac[l + m]) * norm0;
  }
}

// Doubles as float pairs (hi = nearest float, lo = nearest float to the
// remainder), interleaved: the layout of the mixed path's ff values.
void split_pairs(const std::vector<double> &d, std::vector<float> &out) {
  out.resize(2 * d.size());
  for (size_t i = 0; i < d.size(); i++) {
    const float hi = (float)d[i];
    out[2 * i] = hi;
    out[2 * i + 1] = std::isfinite(hi) ? (float)(d[i] - (double)hi) : 0.0f;
  }
}

// Taylor coefficients D^k K_l(z_i)/k!, k = 0..5, of every table point: the
// k-th derivative rows follow from the (k-1)-th by the recurrence of
// src/bessel.c:195-212; row l of the 5th derivative needs rows up to l+5.
void bessel_horner(HostTables &t) {
  const int W = t.tabL + 1, N = t.besselN + 1, HL = t.tabL - 5;
  static const double invfact[6] = {1.0, 1.0, 0.5, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0};
  t.besselHL = HL;
  t.besselH.assign((size_t)N * (HL + 1) * 6, 0.0);
  std::vector<double> d(W + 1), prev(W + 1);
  for (int i = 0; i < N; i++) {
    for (int l = 0; l < W; l++) d[l] = t.besselT[(size_t)i * W + l];
    double *c = &t.besselH[(size_t)i * (HL + 1) * 6];
    for (int l = 0; l <= HL; l++) c[l * 6] = d[l];
    for (int k = 1; k <= 5; k++) {
      int top = t.tabL - k;
      for (int j = 0; j <= top + 1; j++) prev[j] = d[j];
      d[0] = prev[1] - prev[0];
      for (int j = 1; j <= top; j++) d[j] = t.besselC[j] * (prev[j - 1] - prev[j + 1]) - prev[j] + prev[j + 1];
      for (int l = 0; l <= HL; l++) c[l * 6 + k] = d[l] * invfact[k];
    }
  }
  const double h = t.besselN / 16;  // integer division, as src/bessel.c:138-143
  t.besselZ.resize(N);
  for (int i = 0; i < N; i++) t.besselZ[i] = i / h;
  const int AS = HL + 1 < 6 ? 6 : HL + 1;
  t.besselA.assign((size_t)(HL + 1) * AS, 0.0);
  for (int l = 0; l <= HL; l++) {
    double f = l * (l + 1.0), ifac = 1.0;
    t.besselA[(size_t)l * AS] = 1.0;
    for (int i = 1; i <= l; i++) {
      ifac *= i;
      t.besselA[(size_t)l * AS + i] = f / ifac;
      f *= (double)(l + i + 1) * (l - i);
    }
  }
  split_pairs(t.besselH, t.besselHf);
  split_pairs(t.besselA, t.besselAf);
  split_pairs(t.besselZ, t.besselZf);
}

void used_triples(int la, int lb, int l, std::vector<int> &out) {
  int n1 = la + l + 1, n2 = lb + l + 1, n3 = la + lb + 1;
  std::vector<char> used((size_t)n1 * n2 * n3, 0);
  for (int alpha = 0; alpha <= la; alpha++) {
    int ll1 = l - alpha, p1 = (alpha + l) % 2;
    if (p1 > ll1) ll1 = p1;
    for (int beta = 0; beta <= lb; beta++) {
      int ll2 = l - beta, p2 = (beta + l) % 2;
      if (p2 > ll2) ll2 = p2;
      for (int l1 = ll1; l1 <= la + l; l1 += 2)
        for (int l2 = ll2; l2 <= lb + l; l2 += 2) used[((size_t)l1 * n2 + l2) * n3 + alpha + beta] = 1;
    }
  }
  out.clear();
  for (int l1 = 0; l1 < n1; l1++)
    for (int l2 = 0; l2 < n2; l2++)
      for (int l3 = 0; l3 < n3; l3++)
        if (used[((size_t)l1 * n2 + l2) * n3 + l3]) out.push_back(l1 | (l2 << 8) | (l3 << 16));
}

}  // namespace ecpgb

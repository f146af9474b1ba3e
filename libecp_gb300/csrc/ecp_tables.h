// ecp_tables.h -- init-time tables of the ECP engine (host side, FP64).
//
// Everything here depends only on the job's maxima (basis l, ECP L), the
// large-grid order, the quadrature tolerance and the caller's accuracy, never
// on geometry or exponents.  It is the counterpart of what libECP_init builds
// (src/libecp.c:130-198 of chrr/libECP): factorials, the Cartesian ordering,
// the cart->sph and poly->sph matrices, the two Gauss-Chebyshev grids with
// their level schedules, the Bessel table and the angular table Omega.  The
// engine builds a TableSet once per distinct key and keeps it resident on the
// device.
#pragma once
#include <cstdint>
#include <vector>

namespace ecpgb {

// Cartesian / spherical index helpers (libint order; src/dimensions.h:18-37).
constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
constexpr int ncum(int l) { return (l + 1) * (l + 2) * (l + 3) / 6; }
constexpr int nsph(int l) { return (l + 1) * (l + 1); }

// Largest angular momenta the kernels are compiled for.
constexpr int kMaxLBasis = 4;   // basis shells s..g
constexpr int kMaxLEcp = 5;     // ECP channels
constexpr int kMaxTab = kMaxLEcp + kMaxLBasis + 6 + 2;  // Bessel rows

// Level schedule of a nested Gauss-Chebyshev rule.  `slot` lists the
// abscissa indices in the order the adaptive integrator visits them: the
// head (PS93: mid, lower, upper; PSM92: mid), then for every level its
// (lower, upper) pairs.  lvEnd[k] is the slot index one past level k.
struct Schedule {
  int order = 0;
  int headCount = 0;             // 3 for PS93, 1 for PSM92
  int nLevels = 0;
  std::vector<int> lvEnd;        // size nLevels, in slots (pairs count as 2 slots)
  std::vector<int> lvJ;          // PS93 one-/two-point switch per level
  std::vector<int> lvN;          // n after the level
  std::vector<int> slot;         // abscissa index per slot
};

struct TableKey {
  int maxLECP, maxLBS, largeGridOrder;
  double tolerance, accuracy;
  // a caller's Cartesian order (libECP_init's shellOrdering): exponent
  // triples of shells l = 0, 1, ... in the caller's order; empty = libint's
  std::vector<int> ordering;
  // the tables do not depend on the quadrature tolerance
  bool operator==(const TableKey &o) const {
    return maxLECP == o.maxLECP && maxLBS == o.maxLBS && largeGridOrder == o.largeGridOrder &&
           accuracy == o.accuracy && ordering == o.ordering;
  }
};

struct HostTables {
  TableKey key{};
  int maxLECP = 0, maxLBS = 0, maxAlpha = 0, maxLambda = 0;
  int tmDim = 0;        // Cartesian/spherical table rank (>= 2*maxLBS)
  int nk = 0;           // rows of the r^k U_l table (>= la+lb+1 for all pairs)
  int nF = 0;           // rows of the F table (maxLECP - 1 + maxLBS + 1)
  int tabL = 0;         // Bessel table rows - 1
  int besselN = 1600;
  std::vector<double> fac, dfac;
  std::vector<int> ijk;          // 3 ints per Cartesian function up to tmDim
  std::vector<int> ijkIndex;     // (tmDim+1)^3
  std::vector<double> cart2sph;  // blocks [l][m][c]
  std::vector<double> poly2sph;  // [ncum(tmDim)][nsph(tmDim)]
  std::vector<double> xs, ws;    // small grid (PS93 128 -> 383 points, KK-mapped)
  std::vector<double> xl, wl;    // large grid (PSM92, raw on (-1,1))
  Schedule s93, s92;
  std::vector<double> besselT;   // transposed Bessel table [i][l], (N+1) x (tabL+1)
  std::vector<double> besselC;   // C[l] = l/(2l+1)
  // Taylor coefficients of K_l about every table point, [i][l][k], k = 0..5:
  // D^k K_l(z_i) / k!, the derivatives from the reference's recurrence
  // (src/bessel.c:195-212), for l <= besselHL.  K_l(z_i + dz) is then one
  // Horner pass of five multiply-adds per row.
  std::vector<double> besselH;
  int besselHL = 0;
  // The large-argument branch (z >= 16, src/bessel.c:170-190) as a polynomial:
  // K_l(z) = a * sum_i besselA[l][i] (-a)^i with a = 1/(2z), i <= l, row stride
  // max(besselHL + 1, 6), zero beyond i = l.  The coefficients are the integers (l+i)!/((l-i)! i!), the
  // reference's running product divided by i!, so they are exact in FP64.
  std::vector<double> besselA;
  // mixed-precision path: the tables above split into float pairs (hi, lo)
  // with hi + lo = the double to 48 bits (ecp_ff.h), interleaved
  std::vector<float> besselHf, besselAf, besselZf, xlf, wlf;
  std::vector<double> besselZ;   // table abscissae z_i = i / (besselN / 16), the reference's division
  // Normalisation of the real spherical harmonics, [l][m] for l, m <= tmDim:
  // sqrt((2l+1)/(2 pi)) and sqrt((l-m)!/(l+m)!) times that, computed as
  // src/spherical_harmonics.c:236-243 does.
  std::vector<double> shNorm;
  std::vector<double> omega;     // [nsph(maxLECP)][nsph(maxLambda)][ncum(maxAlpha)]
  int omD1 = 0, omD2 = 0;
  int status = 0;                // 0 ok, 1 Bessel series did not converge, 3 sizes out of range
};

// Builds every table for the key.  status != 0 reports a failure.
void build_tables(const TableKey &key, HostTables &t);
void bessel_horner(HostTables &t);
void split_pairs(const std::vector<double> &d, std::vector<float> &out);

// Used triples (l1, l2, l3) of the type-2 radial table for one (la, lb, l):
// exactly those the angular linking of calcGamma (src/type2.c:583-623) reads.
void used_triples(int la, int lb, int l, std::vector<int> &out /* packed l1|l2<<8|l3<<16 */);

}  // namespace ecpgb

// ecp_fp64.cu -- FP64 kernels of the drop-in path for sm_103a.
//
// Compiled with --fmad=false: every multiply and add rounds separately, as
// the reference's C does, so the adaptive quadratures see the same partial
// sums and take the same convergence decisions.
//
// Pipeline of one job (one stream, in order):
//   k_radius        shell radius by Newton (src/util.c:134-192), per shell
//   k_centre        U_l on the small grid, potential screening, r^k U_l
//                   table, local channel (src/type2.c:185-219,
//                   src/libecp.c:268-271), per ECP centre
//   k_centre_atom   rAC, unit-sphere polynomials, real spherical harmonics and
//                   the angular contraction (src/angular_integrals.c:105-142,
//                   src/util.c:215-243), per (centre, atom)
//   k_shell_F       basis-set screening window and F table
//                   (src/type2.c:149-180, :223-310), per (centre, shell)
//   k_unit          one CTA per (centre, shell pair) unit: type-1 block
//                   (src/type1.c:95-302), type-2 block (src/type2.c:337-631),
//                   binomial shift (src/util.c:247-334)
//   k_scatter       upper-triangle accumulation into the AO matrix
//                   (src/getIntegrals.c:23-43), per shell pair
#include <cuda_runtime.h>

#include <climits>
#include <cmath>

#include "ecp_device.cuh"

namespace ecpgb {

// ------------------------------------------------------------- small kernels

__global__ void k_radius(DevJob J) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= J.nShells) return;
  const double *a = J.primA + J.shP[s], *d = J.primD + J.shP[s];
  double zeta = a[0], c = fabs(d[0]);
  for (int i = 1; i < J.shK[s]; i++)
    if (a[i] < zeta && d[i] != 0.0) { zeta = a[i]; c = fabs(d[i]); }
  double r = gto_radius(c, zeta, J.shL[s], 1.0E-14);
  if (r < 0) atomicOr(&J.errWord[1], 1);
  J.radius[s] = r < 0 ? -1.0 : sqrt(r);
}

__global__ void __launch_bounds__(128) k_centre(DevJob J) {
  extern __shared__ double sU[];  // (L+1) x 383
  __shared__ int sEnd[kMaxLEcp + 1];
  __shared__ int sBest;
  const int c = blockIdx.x, L = J.ctrL[c], O = kSmallOrder;
  for (int n = threadIdx.x; n < O; n += blockDim.x) {
    double r = J.xSmall[n];
    for (int l = 0; l <= L; l++) sU[l * O + n] = eval_ecp(J, c, l, r);
  }
  __syncthreads();
  int end = O - 1;
  for (int l = 0; l < L; l++) {
    if (threadIdx.x == 0) sBest = -1;
    __syncthreads();
    int best = -1;
    for (int i = threadIdx.x; i <= end; i += blockDim.x)
      if (fabs(sU[l * O + i]) > 1.0E-14) best = i;
    if (best >= 0) atomicMax(&sBest, best);
    __syncthreads();
    end = sBest;
    if (threadIdx.x == 0) sEnd[l] = end;
    __syncthreads();
  }
  const int LE = J.maxLECP > 0 ? J.maxLECP : 1, nk = J.nk;
  for (int n = threadIdx.x; n < O; n += blockDim.x) {
    double r = J.xSmall[n];
    double *dst = J.utab + ((size_t)c * O + n) * LE * nk;
    for (int l = 0; l < LE; l++) {
      double v = (l < L && n <= sEnd[l]) ? sU[l * O + n] : 0.0;
      bool live = (l < L && n <= sEnd[l]);
      for (int k = 0; k < nk; k++) {
        dst[l * nk + k] = live ? v : 0.0;
        v = v * r;
      }
    }
    J.uL[(size_t)c * O + n] = sU[L * O + n];
  }
  if (threadIdx.x == 0) J.gridEnd[c] = end;
}

__global__ void __launch_bounds__(64) k_centre_atom(DevJob J) {
  __shared__ double rsh[169];
  __shared__ double g[4];
  const int A = blockIdx.x, c = blockIdx.y;
  const int C = J.ctrAtom[c];
  // the atom's largest l, plus the derivative order whose shifts raise it
  // (src/libecp.c:285-286, :292-293)
  const int lA = J.atomMaxL[A] + (J.deriv > 0 ? J.deriv : 0), lmax = J.maxLECP - 1 + lA;
  const size_t ca = (size_t)c * J.nAtoms + A;
  if (threadIdx.x == 0) {
    const double *rC = J.geom + 3 * C, *rA = J.geom + 3 * A;
    double x = rC[0] - rA[0], y = rC[1] - rA[1], z = rC[2] - rA[2];
    double v[3] = {rA[0] - rC[0], rA[1] - rC[1], rA[2] - rC[2]}, S[3];
    g[0] = v[0]; g[1] = v[1]; g[2] = v[2];
    g[3] = sqrt(x * x + y * y + z * z);
    for (int i = 0; i < 4; i++) J.cgeo[ca * 4 + i] = g[i];
    to_spherical(v, S);
    if (lmax >= 0) real_sph(J, lmax, S[1], S[2], rsh);
    // (-x)^i (-y)^j (-z)^k, i+j+k <= lA (src/util.c:215-243)
    int D = J.uspD;
    double *t = J.usp + ca * D * D * D;
    for (int i = 0; i < D * D * D; i++) t[i] = 0.0;
    double px = 1.0, py = 1.0, pz = 1.0;
    for (int i = 0; i <= lA; i++) {
      px = (i == 0) ? 1.0 : -px * v[0];
      for (int j = 0; j <= lA - i; j++) {
        py = (j == 0) ? 1.0 : -py * v[1];
        for (int k = 0; k <= lA - i - j; k++) {
          pz = (k == 0) ? 1.0 : -pz * v[2];
          t[(i * D + j) * D + k] = px * py * pz;
        }
      }
    }
  }
  __syncthreads();
  if (lmax < 0) return;
  const int nlm = J.maxLECP * J.maxLECP, ncA = NCUM(lA);
  const int inc1 = J.omD2, inc2 = J.omD1 * J.omD2;
  const int total = (lmax + 1) * nlm * ncA;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    int cart = e % ncA, rest = e / ncA, lm = rest % nlm, lam = rest / nlm;
    double v = 0.0;
    for (int mu = 0; mu < 2 * lam + 1; mu++)
      v += rsh[lam * lam + mu] * J.omega[(size_t)lm * inc2 + (lam * lam + mu) * inc1 + cart];
    J.ang[((ca * J.angLam + lam) * J.angLM + lm) * J.angC + cart] = v;
  }
}

__global__ void __launch_bounds__(128) k_shell_F(DevJob J) {
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
          bessel_eval(J, lmaxA, 2.0 * zeta * dAC * r, K, 1);
          double e = dAC - r;
          e = exp(-zeta * e * e);
          for (int i = 0; i <= lmaxA; i++) acc[i] += da * K[i] * e;
        }
      }
      for (int i = 0; i < nF; i++) F[(size_t)n * nF + i] = acc[i];
    }
  }
}

// ------------------------------------------------------------ unit kernel

struct UnitShared {
  double sS, sTh, sPh;
  int nb;            // break index of the current large-grid primitive pair
  int anyFail, nFail, allDone, failed;
  int ppBreak[kMaxContraction * kMaxContraction];
  int failIdx[kMaxWalkers];
  unsigned failMask[64];
};

// One (pair, centre) unit per CTA.
__global__ void __launch_bounds__(kUnitThreads, 1) k_unit(DevJob J) {
  extern __shared__ double sm[];
  __shared__ UnitShared S;
  const long long u = blockIdx.x;
  const int c = (int)(u / J.nPairs), pr = (int)(u % J.nPairs);
  const int sa = J.pairA[pr], sb = J.pairB[pr], tid = threadIdx.x, NT = blockDim.x;
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
  const UnitSmem Lm = unit_smem_layout(J.maxLBS, J.maxLECP, J.nF);
  const int A = J.shAtom[sa], B = J.shAtom[sb], la = J.shL[sa] + sh.a, lb = J.shL[sb] + sh.b;
  const int lpa = sh.lpa, lpb = sh.lpb, pa0 = sh.a > 0 ? sh.a : 0, pb0 = sh.b > 0 ? sh.b : 0;
  const int lab = la + lb, nA = 2 * J.maxLBS + 1, LE = J.maxLECP > 0 ? J.maxLECP : 1;
  const int Lc = J.ctrL[c], nca = NCUM(la), ncb = NCUM(lb);
  const int Os = kSmallOrder, OL = J.largeOrder;
  const size_t cA = (size_t)c * J.nAtoms + A, cB = (size_t)c * J.nAtoms + B;
  const double *gA = J.cgeo + cA * 4, *gB = J.cgeo + cB * 4;
  const double dAC = gA[3], dBC = gB[3];
  const double *pzA = J.primA + J.shP[sa], *pcA = J.primD + J.shP[sa];
  const double *pzB = J.primA + J.shP[sb], *pcB = J.primD + J.shP[sb];
  const int Na = J.shK[sa], Nb = J.shK[sb];
  double *chi = sm + Lm.chi, *Jsh = sm + Lm.J, *rsh = sm + Lm.rsh, *Q = sm + Lm.Q;
  double *K1 = sm + Lm.K1, *R1 = sm + Lm.R1, *EX1 = sm + Lm.EX1, *U1 = sm + Lm.U1;
  double *ck = sm + Lm.ck;
  const int CS = Lm.ckStride;
  Walk W{sm + Lm.st, sm + Lm.st + Lm.qItems, sm + Lm.st + 2 * Lm.qItems, sm + Lm.st + 3 * Lm.qItems,
         nullptr};
  __shared__ int sDone[kMaxWalkers];
  W.done = sDone;
  double *out1 = J.out + (size_t)c * J.centreStride + J.pairOff[pr];
  double *out2 = out1 + NCART(lpa) * NCART(lpb);
  const double tol = J.tol;
  if (tid == 0) S.failed = 0;

  // --------------------------------------------------------------- type 1
  for (int e = tid; e < nca * ncb; e += NT) chi[e] = 0.0;
  const int nq1 = [&] { int t = 0; for (int l1 = 0; l1 <= lab; l1++) t += l1 / 2 + 1; return t; }();
  for (int pp = 0; pp < Na * Nb; pp++) {
    const double za = pzA[pp / Nb], zb = pzB[pp % Nb];
    const double ca = zeta_times(pcA[pp / Nb], za, pa0), cb = zeta_times(pcB[pp % Nb], zb, pb0);
    if (tid == 0) {
      double P[3], Sp[3];
      for (int i = 0; i < 3; i++) P[i] = 2.0 * (za * gA[i] + zb * gB[i]);
      to_spherical(P, Sp);
      S.sS = Sp[0]; S.sTh = Sp[1]; S.sPh = Sp[2];
      real_sph(J, lab, Sp[1], Sp[2], rsh);
      S.anyFail = 0;
    }
    for (int e = tid; e < (lab + 1) * (lab + 1); e += NT) Q[e] = 0.0;
    __syncthreads();
    const double s = S.sS, z = -za - zb;
    const double zd2 = -za * dAC * dAC - zb * dBC * dBC;
    for (int n = tid; n < Os; n += NT) {
      double *Kn = K1 + n * nA, *Rn = R1 + n * nA;
      if (n >= ws && n < we) {
        double r = J.xSmall[n], e = (z * r + s) * r;
        EX1[n] = (e >= J.lnAcc1) ? exp(e) : 0.0;
        U1[n] = J.uL[(size_t)c * Os + n];
        bessel_eval(J, lab, s * r, Kn, 1);
        Rn[0] = 1.0;
        for (int l = 1; l <= lab; l++) Rn[l] = r * Rn[l - 1];
      } else {  // the reference's zero-initialised buffers
        EX1[n] = 1.0;
        U1[n] = 0.0;
        for (int l = 0; l <= lab; l++) { Kn[l] = 0.0; Rn[l] = 0.0; }
      }
    }
    __syncthreads();
    const double C1 = ca * cb * exp(zd2);
    for (int q = tid; q < nq1; q += NT) {
      int l1 = 0, rem = q;
      while (rem >= l1 / 2 + 1) { rem -= l1 / 2 + 1; l1++; }
      int l2 = l1 - 2 * rem;
      double res;
      bool ok = ps93_walk(J.wSmall, ws, we, tol, 0.0,
                          [&](int n) { return C1 * R1[n * nA + l1] * U1[n] * K1[n * nA + l2] * EX1[n]; },
                          res);
      if (ok) Q[l1 * (lab + 1) + l2] += res;
      else { S.failIdx[atomicAdd(&S.anyFail, 1)] = l1 | (l2 << 8); }
    }
    __syncthreads();
    if (S.anyFail > 0) {
      // --- large-grid fallback with the Gaussian prefactor regrouped
      //     (src/type1.c:149-196): FM06 map, break at the first point past
      //     both centres whose exponent is below the screen, PSM92.
      const int nf = S.anyFail;
      const double C2 = ca * cb, zp = za + zb, Pm = (za * dAC + zb * dBC) / zp;
      const double sigma = 1.0 / sqrt(zp), t0 = Pm - 7.0 * sigma;
      const double rmin = (t0 > 0.0) ? t0 : 0.0, rmax = Pm + 9.0 * sigma;
      const double i1 = 0.5 * (rmax - rmin), i2 = 0.5 * (rmax + rmin);
      if (tid == 0) S.nb = OL;
      __syncthreads();
      int best = OL;
      for (int n = tid; n < OL; n += NT) {
        double r = i1 * J.xLarge[n] + i2, e = (z * r + s) * r + zd2;
        if (r > dAC && r > dBC && e < J.lnAcc1) { best = n; break; }
      }
      if (best < OL) atomicMin(&S.nb, best);
      for (int q = tid; q < nf; q += NT) { W.I[q] = 0; W.p[q] = 0; W.q[q] = 0; W.res[q] = 0; W.done[q] = 0; }
      __syncthreads();
      const int nb = S.nb, end = nb - 1;
      const int nSlots = OL;
      for (int s0 = 0; s0 < nSlots;) {
        int s1 = s0 == 0 ? 1 + 2 * kChunkPairs : s0 + 2 * kChunkPairs;
        if (s1 > nSlots) s1 = nSlots;
        for (int pos = s0 + tid; pos < s1; pos += NT) {
          // index differs across the warp: the global copy (constant reads serialise)
          int n = J.s92 ? __ldg(J.s92 + pos) : c92_slot[pos];
          double *e = ck + (pos - s0) * CS;  // w, ex, vis, U, R[nA], K[nA]
          double *eR = e + 4, *eK = e + 4 + nA;
          bool upper = (pos > 0) && ((pos - 1) & 1);
          e[0] = J.wLarge[n] * i1;
          e[2] = (!upper || n <= end) ? 1.0 : 0.0;
          if (n < nb) {
            double r = i1 * J.xLarge[n] + i2, ex = (z * r + s) * r + zd2;
            if (ex >= J.lnAcc1) {
              e[1] = exp(ex);
              bessel_eval(J, lab, s * r, eK, 1);
              e[3] = eval_ecp(J, c, Lc, r);
              eR[0] = 1.0;
              for (int l = 1; l <= lab; l++) eR[l] = r * eR[l - 1];
            } else {
              e[1] = 0.0;
            }
          } else if (n == nb || upper) {
            e[1] = 0.0;
          } else {
            // Beyond the break the reference integrates what its buffers
            // still hold from the small-grid stage: exponent and U_L at the
            // same index, r^l and K_l at the same flat offset of a buffer
            // written with the small grid's row stride.
            e[1] = n < Os ? EX1[n] : 1.0;
            e[3] = n < Os ? U1[n] : 0.0;
            for (int l = 0; l <= lab; l++) {
              int f = l * OL + n, lr = f / Os, nr = f % Os;
              eR[l] = lr <= lab ? R1[nr * nA + lr] : 0.0;
              eK[l] = lr <= lab ? K1[nr * nA + lr] : 0.0;
            }
          }
        }
        __syncthreads();
        for (int q = tid; q < nf; q += NT) {
          if (W.done[q]) continue;
          int l1 = S.failIdx[q] & 255, l2 = S.failIdx[q] >> 8;
          double I = W.I[q], p = W.p[q], qq = W.q[q];
          int done = 0;
          double res = 0;
          auto val = [&](int pos) {
            const double *e = ck + (pos - s0) * CS;
            if (e[1] == 0.0) return 0.0;  // exponent below the screen: integrand 0
            return e[0] * (C2 * e[4 + l1] * e[3] * e[4 + nA + l2] * e[1]);
          };
          int pos = s0;
          if (pos == 0) { I = val(0); p = I; pos = 1; }
          while (pos < s1 && !done) {
            int k = level_of(pos);
            int lvStart = k == 0 ? 1 : c92_lvEnd[k - 1];
            if (pos == lvStart) { qq = 2 * p; p = 2 * I; }
            double T = 0.0;
            T += val(pos);
            const double *eh = ck + (pos + 1 - s0) * CS;
            if (eh[2] != 0.0) T += val(pos + 1);
            I += T;
            pos += 2;
            if (pos == c92_lvEnd[k]) {
              double N = c92_lvN[k] + 1.0, ee = I - p;
              if (16 * ee * ee <= 3 * N * fabs(I - qq) * tol) { res = 16 * I / (3 * N); done = 1; }
            }
          }
          W.I[q] = I; W.p[q] = p; W.q[q] = qq;
          if (done) { W.res[q] = res; W.done[q] = 1; }
        }
        if (tid == 0) S.allDone = 1;
        __syncthreads();
        for (int q = tid; q < nf; q += NT)
          if (!W.done[q]) S.allDone = 0;
        __syncthreads();
        if (S.allDone) break;
        s0 = s1;
      }
      // out of levels: the full-grid estimate stands and the unit is flagged
      const double Nlast = c92_lvN[c92_nLevels - 1] + 1.0;
      for (int q = tid; q < nf; q += NT) {
        int l1 = S.failIdx[q] & 255, l2 = S.failIdx[q] >> 8;
        if (W.done[q]) Q[l1 * (lab + 1) + l2] += W.res[q];
        else { Q[l1 * (lab + 1) + l2] += 16 * W.I[q] / (3 * Nlast); S.failed = kUnitWarnType1; }
      }
      __syncthreads();
    }
    // chi[i][j] += sum_l (sum_m S_lm poly2sph) Q[lmax][l]  (src/type1.c:266-295)
    const int dd = J.tmDim + 1, tmW = (J.tmDim + 1) * (J.tmDim + 1);
    for (int e = tid; e < nca * ncb; e += NT) {
      int i = e / ncb, j = e % ncb;
      const int *ei = J.ijk + 3 * i, *ej = J.ijk + 3 * j;
      int lx = ei[0] + ej[0], ly = ei[1] + ej[1], lz = ei[2] + ej[2], lmax = lx + ly + lz;
      int p = J.ijkIdx[(lx * dd + ly) * dd + lz];
      double acc = chi[e];
      for (int l = lmax; l >= 0; l -= 2) {
        double factor = 0.0;
        for (int m = 0; m < 2 * l + 1; m++) factor += rsh[l * l + m] * J.p2s[(size_t)p * tmW + l * l + m];
        acc += factor * Q[lmax * (lab + 1) + l];
      }
      chi[e] = acc;
    }
    __syncthreads();
  }

  // binomial shift onto A and B (src/util.c:247-334); J then I
  auto poly_shift = [&](double norm, double *dst) {
    const int D = J.uspD, dd = J.tmDim + 1, nta = NCART(lpa), ntb = NCART(lpb);
    const double *uA = J.usp + cA * D * D * D, *uB = J.usp + cB * D * D * D;
    for (int e = tid; e < nta * ncb; e += NT) {
      int c1 = e / ncb, q = e % ncb;
      const int *ex = J.ijk + 3 * (NCUM(lpa - 1) + c1);
      double v = 0.0;
      for (int x = 0; x <= ex[0]; x++) {
        double bx = binom(J.fac, ex[0], x);
        for (int y = 0; y <= ex[1]; y++) {
          double by = bx * binom(J.fac, ex[1], y);
          for (int zz = 0; zz <= ex[2]; zz++) {
            double bz = by * binom(J.fac, ex[2], zz);
            double factor = bz * uA[((ex[0] - x) * D + (ex[1] - y)) * D + (ex[2] - zz)];
            if (fabs(factor) <= J.acc) continue;
            int r = J.ijkIdx[(x * dd + y) * dd + zz];
            v += factor * chi[r * ncb + q];
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
        double bx = binom(J.fac, ex[0], x);
        for (int y = 0; y <= ex[1]; y++) {
          double by = bx * binom(J.fac, ex[1], y);
          for (int zz = 0; zz <= ex[2]; zz++) {
            double bz = by * binom(J.fac, ex[2], zz);
            double factor = bz * uB[((ex[0] - x) * D + (ex[1] - y)) * D + (ex[2] - zz)];
            if (fabs(factor) <= J.acc) continue;
            factor *= norm;
            int r = J.ijkIdx[(x * dd + y) * dd + zz];
            v += factor * Jsh[c1 * ncb + r];
          }
        }
      }
      dst[e] = v;
    }
    __syncthreads();
  };
  const double norm1 = 4.0 * kPi, norm2 = norm1 * norm1;
  poly_shift(norm1, out1);

  // --------------------------------------------------------------- type 2
  const int nF = J.nF, LBE = J.maxLBS + LE;
  double *Fa = sm + Lm.Fa, *Fb = sm + Lm.Fb, *T = sm + Lm.T;
  // F tables of the derivative runs max(0, shift) (src/type2.c:563-564)
  const int nRuns = J.nRuns > 0 ? J.nRuns : 1;
  const double *gFa = J.F + (((size_t)c * J.nShells + sa) * nRuns + pa0) * Os * nF;
  const double *gFb = J.F + (((size_t)c * J.nShells + sb) * nRuns + pb0) * Os * nF;
  for (int e = tid; e < Os * nF; e += NT) { Fa[e] = gFa[e]; Fb[e] = gFb[e]; }
  for (int e = tid; e < LE * LBE * LBE * nA; e += NT) T[e] = 0.0;
  for (int e = tid; e < nca * ncb; e += NT) chi[e] = 0.0;
  for (int e = tid; e < 64; e += NT) S.failMask[e] = 0;
  if (tid == 0) S.nFail = 0;
  __syncthreads();
  const double *Ut = J.utab + (size_t)c * Os * LE * J.nk;
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
  for (int q = tid; q < nItems; q += NT) {
    int l, l1, l2, l3;
    item(q, l, l1, l2, l3);
    const int nk = J.nk;
    double res;
    bool ok = ps93_walk(J.wSmall, ws, we, tol, 0.0,
                        [&](int n) {
                          return Fa[n * nF + l1] * Fb[n * nF + l2] * Ut[((size_t)n * LE + l) * nk + l3];
                        },
                        res);
    if (ok) T[tidx(l, l1, l2, l3)] = res;
    else { atomicOr(&S.failMask[q >> 5], 1u << (q & 31)); atomicAdd(&S.nFail, 1); }
  }
  __syncthreads();
  if (S.nFail > 0) {
    // --- per-primitive-pair large-grid fallback (src/type2.c:418-528)
    const int NP = Na * Nb, laC = la + Lc - 1, lbC = lb + Lc - 1;
    // break index of every primitive pair: the first point past both
    // centres whose exponent is below the screen; monotone in the index
    // there, so a bisection finds it.
    for (int k = tid; k < NP; k += NT) {
      double za = pzA[k / Nb], zb = pzB[k % Nb], zp = za + zb, Pm = (za * dAC + zb * dBC) / zp;
      double sigma = 1.0 / sqrt(zp), t0 = Pm - 7.0 * sigma;
      double rmin = (t0 > 0.0) ? t0 : 0.0, rmax = Pm + 9.0 * sigma;
      double i1 = 0.5 * (rmax - rmin), i2 = 0.5 * (rmax + rmin);
      auto pred = [&](int n) {
        double r = i1 * J.xLarge[n] + i2, d1 = dAC - r, d2 = dBC - r;
        double e = -za * d1 * d1 - zb * d2 * d2;
        return r > dAC && r > dBC && e < J.lnAcc2;
      };
      int lo = 0, hi = OL;  // first true in [lo, hi), OL = none
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (pred(mid)) hi = mid; else lo = mid + 1;
      }
      S.ppBreak[k] = lo < OL ? lo : INT_MAX;
    }
    __syncthreads();
    // Failed items, processed kMaxWalkers at a time.
    for (int base = 0; base < nItems; ) {
      if (tid == 0) {
        int nf = 0, q = base;
        for (; q < nItems && nf < kMaxWalkers; q++)
          if (S.failMask[q >> 5] & (1u << (q & 31))) S.failIdx[nf++] = q;
        S.anyFail = nf;
        S.nb = q;  // next base
      }
      __syncthreads();
      const int nf = S.anyFail, nextBase = S.nb;
      for (int k = 0; k < NP; k++) {
        const double za = pzA[k / Nb], ca = pcA[k / Nb], zb = pzB[k % Nb], cb = pcB[k % Nb];
        const double Ck = zeta_times(zeta_times(ca * cb, za, pa0), zb, pb0);
        const double zp = za + zb, Pm = (za * dAC + zb * dBC) / zp;
        const double sigma = 1.0 / sqrt(zp), t0 = Pm - 7.0 * sigma;
        const double rmin = (t0 > 0.0) ? t0 : 0.0, rmax = Pm + 9.0 * sigma;
        const double i1 = 0.5 * (rmax - rmin), i2 = 0.5 * (rmax + rmin);
        const int nb = S.ppBreak[k], end = nb == INT_MAX ? OL - 1 : nb - 1;
        for (int q = tid; q < nf; q += NT) { W.I[q] = 0; W.p[q] = 0; W.q[q] = 0; W.done[q] = 0; }
        __syncthreads();
        for (int s0 = 0; s0 < OL;) {
          int s1 = s0 == 0 ? 1 + 2 * kChunkPairs : s0 + 2 * kChunkPairs;
          if (s1 > OL) s1 = OL;
          for (int pos = s0 + tid; pos < s1; pos += NT) {
            int n = J.s92 ? __ldg(J.s92 + pos) : c92_slot[pos];
            double *e = ck + (pos - s0) * CS;  // w, ex, vis, U[LE], R[nA], Ka[LBE], Kb[LBE]
            double *eU = e + 3, *eR = eU + LE, *eKa = eR + nA, *eKb = eKa + LBE;
            bool upper = (pos > 0) && ((pos - 1) & 1);
            e[0] = J.wLarge[n] * i1;
            e[2] = (!upper || n <= end) ? 1.0 : 0.0;
            // whose tables does index n hold: this pair's if it was reached,
            // else (lower half only) the last earlier pair that reached it
            int owner = -1;
            if (n < nb) owner = k;
            else if (n != nb && !upper) {
              for (int j = k - 1; j >= 0; j--)
                if (S.ppBreak[j] >= n) { owner = j; break; }
              if (owner >= 0 && S.ppBreak[owner] == n) owner = -1;
            }
            e[1] = 0.0;
            if (owner >= 0) {
              const double zaj = pzA[owner / Nb], zbj = pzB[owner % Nb];
              double i1j = i1, i2j = i2;
              if (owner != k) {
                double zpj = zaj + zbj, Pj = (zaj * dAC + zbj * dBC) / zpj;
                double sg = 1.0 / sqrt(zpj), tj = Pj - 7.0 * sg;
                double rmn = (tj > 0.0) ? tj : 0.0, rmx = Pj + 9.0 * sg;
                i1j = 0.5 * (rmx - rmn);
                i2j = 0.5 * (rmx + rmn);
              }
              double r = i1j * J.xLarge[n] + i2j, d1 = dAC - r, d2 = dBC - r;
              double ex = -zaj * d1 * d1 - zbj * d2 * d2;
              if (ex >= J.lnAcc2) {
                e[1] = exp(ex);
                for (int l = 0; l < Lc; l++) eU[l] = eval_ecp(J, c, l, r);
                bessel_eval(J, laC, 2.0 * zaj * dAC * r, eKa, 1);
                bessel_eval(J, lbC, 2.0 * zbj * dBC * r, eKb, 1);
                eR[0] = 1.0;
                for (int l = 1; l <= lab; l++) eR[l] = r * eR[l - 1];
              }
            }
          }
          __syncthreads();
          for (int q = tid; q < nf; q += NT) {
            if (W.done[q]) continue;
            int l, l1, l2, l3;
            item(S.failIdx[q], l, l1, l2, l3);
            double I = W.I[q], p = W.p[q], qq = W.q[q];
            int done = 0;
            double res = 0;
            auto val = [&](int pos) {
              const double *e = ck + (pos - s0) * CS;
              if (e[1] == 0.0) return 0.0;  // exponent below the screen: integrand 0
              const double *eU = e + 3, *eR = eU + LE, *eKa = eR + nA, *eKb = eKa + LBE;
              return e[0] * (Ck * eU[l] * eR[l3] * eKa[l1] * eKb[l2] * e[1]);
            };
            int pos = s0;
            if (pos == 0) { I = val(0); p = I; pos = 1; }
            while (pos < s1 && !done) {
              int kk = level_of(pos);
              int lvStart = kk == 0 ? 1 : c92_lvEnd[kk - 1];
              if (pos == lvStart) { qq = 2 * p; p = 2 * I; }
              double Tq = 0.0;
              Tq += val(pos);
              const double *eh = ck + (pos + 1 - s0) * CS;
              if (eh[2] != 0.0) Tq += val(pos + 1);
              I += Tq;
              pos += 2;
              if (pos == c92_lvEnd[kk]) {
                double N = c92_lvN[kk] + 1.0, ee = I - p;
                if (16 * ee * ee <= 3 * N * fabs(I - qq) * tol) { res = 16 * I / (3 * N); done = 1; }
              }
            }
            W.I[q] = I; W.p[q] = p; W.q[q] = qq;
            if (done) { W.res[q] = res; W.done[q] = 1; }
          }
          if (tid == 0) S.allDone = 1;
          __syncthreads();
          for (int q = tid; q < nf; q += NT)
            if (!W.done[q]) S.allDone = 0;
          __syncthreads();
          if (S.allDone) break;
          s0 = s1;
        }
        const double Nlast = c92_lvN[c92_nLevels - 1] + 1.0;
        for (int q = tid; q < nf; q += NT) {
          int l, l1, l2, l3;
          item(S.failIdx[q], l, l1, l2, l3);
          if (W.done[q]) T[tidx(l, l1, l2, l3)] += W.res[q];
          else {
            T[tidx(l, l1, l2, l3)] += 16 * W.I[q] / (3 * Nlast);
            if (S.failed == 0) S.failed = kUnitWarnType2;
          }
        }
        __syncthreads();
      }
      base = nextBase;
      __syncthreads();
    }
  }
  // gamma[p][q] += sum_l sum_{lambda1, lambda2} (sum_m OmA OmB) T  (src/type2.c:583-623)
  {
    const double *angA = J.ang + cA * J.angLam * J.angLM * J.angC;
    const double *angB = J.ang + cB * J.angLam * J.angLM * J.angC;
    const int LM = J.angLM, AC = J.angC;
    for (int e = tid; e < nca * ncb; e += NT) {
      int pidx = e / ncb, qidx = e % ncb;
      int alpha = 0;
      while (NCUM(alpha) <= pidx) alpha++;
      int beta = 0;
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
              factor += angA[((size_t)l1 * LM + l * l + m) * AC + pidx] *
                        angB[((size_t)l2 * LM + l * l + m) * AC + qidx];
            tmp += factor * T[tidx(l, l1, l2, alpha + beta)];
          }
        g += tmp;
      }
      chi[e] = g;
    }
  }
  __syncthreads();
  poly_shift(norm2, out2);
  if (tid == 0) {
    J.status[u] = S.failed ? S.failed : kUnitDone;
    if (S.failed) atomicMin(&J.errWord[0], (int)u);
  }
}

// AO matrix, upper triangle: per element the centres' type-1 and type-2
// contributions in the reference's order (src/getIntegrals.c:36-42).
__global__ void k_scatter(DevJob J) {
  const int pr = blockIdx.x, sa = J.pairA[pr], sb = J.pairB[pr];
  const int la = J.shL[sa], lb = J.shL[sb], na = NCART(la), nb = NCART(lb);
  const int a0 = J.shAO[sa], b0 = J.shAO[sb];
  for (int e = threadIdx.x; e < na * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    if (a0 + i > b0 + j) continue;
    double acc = 0.0;
    for (int c = 0; c < J.nCentres; c++) {
      long long u = (long long)c * J.nPairs + pr;
      if (J.status[u] == kUnitSkipped) continue;
      const double *o = J.out + (size_t)c * J.centreStride + J.pairOff[pr];
      acc += o[e];
      acc += o[na * nb + e];
    }
    J.mat[(size_t)(a0 + i) * J.dim + b0 + j] += acc;
  }
}

// ------------------------------------------------------------ launchers

int upload_schedules(const int *s93slot, int s93n, const int *s93lvEnd, const int *s93lvJ,
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

int launch_fp64_pipeline(const DevJob &J, cudaStream_t st, size_t smemBytes, cudaEvent_t u0,
                         cudaEvent_t u1) {
  // function attributes are per device; callers hold the engine lock
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    cudaFuncSetAttribute(k_unit, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr[dev] = true;
  }
  if (smemBytes > 200 * 1024) return 3;
  launch_prologue(J, st, true);
  long long nUnits = (long long)J.nCentres * J.nPairs;
  if (u0) record_timing(u0, st);
  if (nUnits > 0) k_unit<<<(unsigned)nUnits, kUnitThreads, smemBytes, st>>>(J);
  if (u1) record_timing(u1, st);
  launch_epilogue(J, st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : kLaunchErrorBase + (int)e;
}

// Per-job stages before and after the unit kernel; shared by both paths
// (the batched path launches its own F-table kernel: withF false).
void launch_prologue(const DevJob &J, cudaStream_t st, bool withF) {
  k_radius<<<(J.nShells + 127) / 128, 128, 0, st>>>(J);
  k_centre<<<J.nCentres, 128, sizeof(double) * kSmallOrder * (kMaxLEcp + 1), st>>>(J);
  k_centre_atom<<<dim3(J.nAtoms, J.nCentres), 64, 0, st>>>(J);
  if (withF) k_shell_F<<<dim3(J.nShells, J.nCentres), 128, 0, st>>>(J);
}

void launch_epilogue(const DevJob &J, cudaStream_t st) {
  // the AO matrix exists for derivative order 0 only (getIntegrals)
  if (J.nPairs > 0 && J.deriv == 0) k_scatter<<<J.nPairs, 128, 0, st>>>(J);
}

}  // namespace ecpgb

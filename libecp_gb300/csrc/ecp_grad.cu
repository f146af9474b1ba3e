// ecp_grad.cu -- device-side consumers of the ECP blocks: the energy
// E = sum_{mu nu} D_{mu nu} V_{mu nu} of a density matrix D and its nuclear
// gradient from the derivative-order-1 blocks, contracted where the blocks
// are (nothing but the result leaves the GPU).
//
// Gradient of one (shell pair a, b; centre C) block.  A Cartesian Gaussian
// g(a) centred on A has d g(a) / d A_k = 2 zeta g(a + 1_k) - a_k g(a - 1_k);
// the reference's shift (+1, 0) blocks already carry the factor zeta
// (src/type1.c:239-246, src/type2.c:456-462), so
//   d<a|U_C|b>/dA_k = 2 P[a + 1_k][b] - a_k M[a - 1_k][b],
// P, M the (type-1 + type-2) blocks of shifts (+1, 0) and (-1, 0), and the
// same on the ket with (0, +1), (0, -1).  The potential moves with C, and
// translational invariance gives d/dC = -(d/dA + d/dB); atom A receives
// d/dA, atom B d/dB and atom C -(d/dA + d/dB).  Where the reference computes
// no block (A = C for a bra shift, B = C for a ket shift, A = B = C, screened
// pairs) the block is zero here, and the missing terms cancel in exactly
// that sum (atom A = C receives -d/dB).
#include <cuda_runtime.h>

#include "ecp_device.cuh"

namespace ecpgb {

// Position of Cartesian function (x, y, z) within its shell (libint order,
// via the cumulative index table).
static __device__ inline int in_shell(const DevJob &J, int x, int y, int z) {
  const int dd = J.tmDim + 1, l = x + y + z;
  return J.ijkIdx[(x * dd + y) * dd + z] - NCUM(l - 1);
}

// One warp per (centre, shell pair): the six contractions D . dV/dA_k,
// D . dV/dB_k, added to the three atoms.  J describes a derivative-order-1
// job: pair entries come in fours, shifts (+1,0), (-1,0), (0,+1), (0,-1).
__global__ void k_grad(DevJob J, const double *D, int ldD, double *grad) {
  const int lane = threadIdx.x & 31;
  const long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int nBase = J.nPairs / 4;
  if (w >= (long long)J.nCentres * nBase) return;
  const int c = (int)(w / nBase), pb = (int)(w % nBase), px = 4 * pb;
  const int sa = J.pairA[px], sb = J.pairB[px], la = J.shL[sa], lb = J.shL[sb];
  const int A = J.shAtom[sa], B = J.shAtom[sb], C = J.ctrAtom[c];
  const int na = NCART(la), nb = NCART(lb), a0 = J.shAO[sa], b0 = J.shAO[sb];
  const double wgt = sa == sb ? 1.0 : 2.0;  // a block off the diagonal stands for its transpose too
  const double *blk[4];
  int rows[4], cols[4];
  for (int k = 0; k < 4; k++) {
    const long long u = (long long)c * J.nPairs + px + k;
    blk[k] = J.status[u] == kUnitSkipped ? nullptr : J.out + (size_t)c * J.centreStride + J.pairOff[px + k];
    const int lpa = la + (k == 0) - (k == 1), lpb = lb + (k == 2) - (k == 3);
    rows[k] = lpa >= 0 ? NCART(lpa) : 0;
    cols[k] = lpb >= 0 ? NCART(lpb) : 0;
  }
  // type-1 + type-2 value of block k at (row, col)
  auto val = [&](int k, int r, int q) {
    const double *b = blk[k];
    if (!b) return 0.0;
    const int n = rows[k] * cols[k];
    return b[r * cols[k] + q] + b[n + r * cols[k] + q];
  };
  double dA[3] = {0, 0, 0}, dB[3] = {0, 0, 0};
  const int *ea = J.ijk + 3 * NCUM(la - 1), *eb = J.ijk + 3 * NCUM(lb - 1);
  for (int e = lane; e < na * nb; e += 32) {
    const int i = e / nb, j = e % nb;
    const double dm = wgt * D[(size_t)(a0 + i) * ldD + b0 + j];
    const int *xa = ea + 3 * i, *xb = eb + 3 * j;
    for (int k = 0; k < 3; k++) {
      int up[3] = {xa[0], xa[1], xa[2]};
      up[k]++;
      double t = 2.0 * val(0, in_shell(J, up[0], up[1], up[2]), j);
      if (xa[k] > 0) {
        up[k] -= 2;
        t -= xa[k] * val(1, in_shell(J, up[0], up[1], up[2]), j);
      }
      dA[k] += dm * t;
      int vp[3] = {xb[0], xb[1], xb[2]};
      vp[k]++;
      double s = 2.0 * val(2, i, in_shell(J, vp[0], vp[1], vp[2]));
      if (xb[k] > 0) {
        vp[k] -= 2;
        s -= xb[k] * val(3, i, in_shell(J, vp[0], vp[1], vp[2]));
      }
      dB[k] += dm * s;
    }
  }
  for (int off = 16; off; off >>= 1)
    for (int k = 0; k < 3; k++) {
      dA[k] += __shfl_down_sync(0xffffffffu, dA[k], off);
      dB[k] += __shfl_down_sync(0xffffffffu, dB[k], off);
    }
  if (lane == 0)
    for (int k = 0; k < 3; k++) {
      atomicAdd(&grad[3 * A + k], dA[k]);
      atomicAdd(&grad[3 * B + k], dB[k]);
      atomicAdd(&grad[3 * C + k], -(dA[k] + dB[k]));
    }
}

// E = sum_{i <= j} (2 - delta_ij) D_ij V_ij over the upper triangle of the AO
// matrix; one CTA, a fixed summation order (deterministic).
__global__ void __launch_bounds__(1024) k_energy(const double *V, int dim, const double *D, int ldD,
                                                 double *E) {
  __shared__ double part[1024];
  double acc = 0.0;
  for (long long e = threadIdx.x; e < (long long)dim * dim; e += blockDim.x) {
    const int i = (int)(e / dim), j = (int)(e % dim);
    if (j < i) continue;
    acc += (i == j ? 1.0 : 2.0) * D[(size_t)i * ldD + j] * V[e];
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *E = part[0];
}

// Real-spherical blocks: S = T(la) B T(lb)^T for both blocks of every
// emitted unit, T the Cartesian -> real spherical matrices of
// src/transformations.c:29-87 ([l][m][c] blocks, in the job's Cartesian
// order).  One CTA per unit; sphOff / sphStride the spherical layout.
__global__ void __launch_bounds__(64) k_to_sph(DevJob J, const double *c2s, const long long *sphOff,
                                               long long sphStride, double *sout) {
  __shared__ double tmp[2 * 15 * 15];
  const long long u = blockIdx.x;
  if (J.status[u] == kUnitSkipped) return;
  const int c = (int)(u / J.nPairs), px = (int)(u % J.nPairs);
  const UnitShift sh = unit_shift(J, px, J.shL[J.pairA[px]], J.shL[J.pairB[px]], 0, 1, 2);
  const int la = sh.lpa, lb = sh.lpb, na = NCART(la), nb = NCART(lb), ma = 2 * la + 1, mb = 2 * lb + 1;
  auto off = [](int l) {
    int o = 0;
    for (int k = 0; k < l; k++) o += (2 * k + 1) * NCART(k);
    return o;
  };
  const double *Ta = c2s + off(la), *Tb = c2s + off(lb);
  const double *src = J.out + (size_t)c * J.centreStride + J.pairOff[px];
  double *dst = sout + (size_t)c * sphStride + sphOff[px];
  for (int t = 0; t < 2; t++) {
    const double *B = src + t * na * nb;
    for (int e = threadIdx.x; e < ma * nb; e += blockDim.x) {  // T(la) B
      const int m = e / nb, j = e % nb;
      double v = 0.0;
      for (int i = 0; i < na; i++) v += Ta[m * na + i] * B[i * nb + j];
      tmp[e] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ma * mb; e += blockDim.x) {  // (T(la) B) T(lb)^T
      const int m = e / mb, n = e % mb;
      double v = 0.0;
      for (int j = 0; j < nb; j++) v += tmp[m * nb + j] * Tb[n * nb + j];
      dst[t * ma * mb + e] = v;
    }
    __syncthreads();
  }
}

void launch_to_sph(const DevJob &J, const double *c2s, const long long *sphOff, long long sphStride,
                   double *sout, cudaStream_t st) {
  const long long n = (long long)J.nCentres * J.nPairs;
  if (n > 0) k_to_sph<<<(unsigned)n, 64, 0, st>>>(J, c2s, sphOff, sphStride, sout);
}

void launch_gradient(const DevJob &J, const double *D, int ldD, double *grad, cudaStream_t st) {
  const long long warps = (long long)J.nCentres * (J.nPairs / 4);
  if (warps <= 0) return;
  const int perBlock = 8;
  k_grad<<<(unsigned)((warps + perBlock - 1) / perBlock), 32 * perBlock, 0, st>>>(J, D, ldD, grad);
}

void launch_energy(const double *V, int dim, const double *D, int ldD, double *E, cudaStream_t st) {
  k_energy<<<1, 1024, 0, st>>>(V, dim, D, ldD, E);
}

}  // namespace ecpgb

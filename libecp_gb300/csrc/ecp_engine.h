// ecp_engine.h -- device-side job description shared by the host driver
// (ecp_engine.cu) and the kernels (ecp_fp64.cu).
//
// HBM layout of one job (all arrays device-resident, FP64 unless noted):
//   inputs      geometry[3*nAtoms]; per shell l, K, first primitive, atom,
//               AO offset; per primitive exponent/coefficient; per ECP centre
//               atom, L, term range; per term l, n, d, a; the pair list in the
//               reference's loop order (A, B>=A, s1, s2).
//   per centre  r^k U_l on the small grid, point-major [383][maxLECP][nk];
//               the local channel U_L [383]; the screened grid end.
//   per centre  rAC, dAC, unit-sphere polynomials and the contracted angular
//   and atom    table [lambda][lm][Cartesian] of src/angular_integrals.c:105.
//   per centre  screening window (start, end, skip) and the F table,
//   and shell   point-major [383][nF], zero outside the window.
//   output      per (centre, pair) unit a type-1 block then a type-2 block,
//               NCART(la) x NCART(lb) each, row-major; a status word per unit;
//               the upper triangle of the AO matrix.
// Units are numbered u = centre * nPairs + pair, i.e. the reference's
// callback order (src/libecp.c:256-397).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ecp_ff.h"

namespace ecpgb {

constexpr int kSmallOrder = 383;       // PS93(128) abscissae
constexpr int kMaxLargeOrder = 4095;   // PSM92 abscissae (largeGridOrder < 8192)
constexpr int kMaxContraction = 16;    // primitives per shell
constexpr int kUnitThreads = 128;      // threads per unit CTA
constexpr int kChunkPairs = 64;        // (lower, upper) pairs per fallback chunk
constexpr int kMaxWalkers = 512;       // large-grid quadratures integrated per pass

// Unit status words.
enum : int {
  kUnitDone = 0,        // both blocks written
  kUnitSkipped = 1,     // screened out: the reference makes no callback
  kUnitWarnType1 = 2,   // written; a type-1 large-grid quadrature ran out of levels
                        // and kept its full-grid estimate (the reference aborts)
  kUnitWarnType2 = 3,   // written; the same for a type-2 quadrature only
};

// Per-class launch settings (ecp_fast.cu): classes (la, lb) with la, lb <= 4.
constexpr int kMaxClasses = 25;
constexpr int kClassSet = 1 << 20;

struct DevJob {
  // sizes
  int nAtoms, nShells, nPrims, nCentres, nPairs, dim;
  int maxLECP, maxLBS, maxLambda, nk, nF, tmDim, tabL, besselN;
  int omD1, omD2;              // omega dims [nsph(maxLECP)][omD1][omD2]
  int angLam, angLM, angC;     // per (centre, atom) angular table dims
  int uspD;                    // unit-sphere polynomial table side (maxLBS + 1)
  int largeOrder;
  double tol, acc, lnAcc1, lnAcc2;
  // inputs
  const double *geom;
  const int *shL, *shK, *shP, *shAtom, *shAO;
  const double *primA, *primD;
  const int *ctrAtom, *ctrL, *ctrT0, *ctrNT;
  const int *termL;
  const double *termN, *termD, *termA;
  const int *pairA, *pairB;
  const int *pairShift;        // derivative shift index of each pair entry (null: none)
  int deriv, nRuns;            // derivative order; F-table runs (1 + order; 0 reads as 1)
  const long long *pairOff;    // value offset of the pair's two blocks within a centre
  long long centreStride;      // values per centre
  // used-triple lists of the type-2 angular linking, per (la, lb, l)
  const int *itemOff, *itemCnt, *items;
  // tables
  const double *xSmall, *wSmall, *xLarge, *wLarge;
  const double *besT, *besC;
  const double *besH;          // Taylor coefficients [i][l <= besHL][6] (batched path)
  const double *besA;          // large-argument polynomial [l][i], stride max(besHL + 1, 6)
  // the level schedules' slot tables in global memory as well, for reads
  // whose index differs across a warp (the __constant__ copies serialise those)
  const int *s93, *s92;
  const short *byN93;          // small-grid slots step by step in ascending point order
  // mixed path: tables as float pairs (ecp_ff.h)
  const ff *besHf, *besAf, *besZf;  // besH, besA, besZ
  const ff *xLf, *wLf;              // large grid abscissae and weights
  const ff *termAf, *termDf;        // ECP term exponents and coefficients
  const double *besZ;          // Bessel table abscissae i / (besselN / 16)
  int besHL;
  const double *shNorm;        // spherical-harmonic normalisation [l][m], side tmDim + 1
  const double *p2s, *fac, *dfac;
  const int *atomMaxL;
  const int *ijk, *ijkIdx;
  const double *omega;
  // per-job work arrays
  double *radius;
  double *utab, *uL;
  int *gridEnd;
  int *win;
  double *F;
  double *cgeo, *usp, *ang;
  double *out;
  int *status;
  double *mat;
  int *errWord;          // [0] first unit with a warning (atomicMin), [1] input error flags
  // batched path: work queue and tuning
  const int *order;              // units by descending estimated cost (null: natural order)
  const int *orderClass;         // units grouped by (la, lb, L) class, by cost within a class
  unsigned long long *queueHead; // next queue position (persistent launch); reset per run
  int gcap;                      // type-1 step-table width cap (doubles per slot per warp)
  int maxNP;                     // most primitive pairs of a shell pair (shared-memory sizing)
  int mixed;                     // 1: the fallbacks' tables and sums in double-single (ecp_ff.h)
  int balance;                   // 1: type-1 groups narrowed so that every warp gets pairs
  int ctaUnits;                  // >0: a persistent CTA takes at most this many units, then exits
  // per-(la, lb)-class type-1 settings (index la * (maxLBS + 1) + lb):
  // 0 = the job's gcap and balance, else kClassSet | gcap | balance << 12
  int classCfg[kMaxClasses];
  unsigned long long *classCycles;  // non-null: clock cycles of each class's units (autotuner)
  // screening stage (batched path): the queue of units that compute blocks
  int *live;                     // live units in queue order (null: no screening stage)
  unsigned long long *liveCount; // their number
  int *screenBlocks;             // per-CTA counts, then offsets, of the screening kernels
};

// Launch configuration of the batched path (picked by the autotuner).
struct FastConfig {
  int queue = 1;   // 1: persistent CTAs pulling units from the work queue; 0: a CTA per unit
  int sorted = 1;  // 1: units by descending estimated cost; 2: class-major; 0: the reference's order
  int gcap = 45;   // type-1 step-table width cap; smaller caps fit more CTAs per SM
  int mixed = 0;   // set from the job's mode (ECPGB_MIXED), not tuned
  int balance = 1; // narrower type-1 groups when a unit has few primitive pairs
  int screen = 1;  // with the queue launch: a screening stage compacts the queue to live units
  // per-(la, lb)-class type-1 cap and balance (DevJob::classCfg); the launch's
  // shared memory is sized by gcap, so a class's cap is at most gcap
  int cls[kMaxClasses] = {};
  unsigned long long *classCycles = nullptr;  // autotuner: per-class cycle counts
};

// Shared-memory layout of the unit kernel (offsets in doubles).
struct UnitSmem {
  int K1, R1, EX1, U1, rsh, Q, chi, J, Fa, Fb, T, st, ck, total;
  int qItems;     // per-thread walker state capacity (items)
  int ckStride;   // doubles per chunk point
};

__host__ __device__ inline UnitSmem unit_smem_layout(int LB, int LE, int nF) {
  UnitSmem s{};
  int LAB = 2 * LB, nA = LAB + 1, nE = LE > 0 ? LE : 1;
  int nc = (LB + 1) * (LB + 2) * (LB + 3) / 6, nct = (LB + 1) * (LB + 2) / 2;
  int o = 0;
  s.chi = o; o += nc * nc;
  s.J = o; o += nct * nc;
  s.rsh = o; o += nA * nA;
  s.Q = o; o += nA * nA;
  int base = o;
  // type-1 phase
  s.K1 = o; o += kSmallOrder * nA;
  s.R1 = o; o += kSmallOrder * nA;
  s.EX1 = o; o += kSmallOrder;
  s.U1 = o; o += kSmallOrder;
  int t1end = o;
  // type-2 phase (overlays the type-1 tables)
  o = base;
  s.Fa = o; o += kSmallOrder * nF;
  s.Fb = o; o += kSmallOrder * nF;
  s.T = o; o += nE * (LB + nE) * (LB + nE) * nA;
  int t2end = o;
  o = t1end > t2end ? t1end : t2end;
  // walker state for large-grid items (I, p, q, result) and chunk tables;
  // failed items beyond kMaxWalkers are integrated in further passes
  s.qItems = kMaxWalkers;
  if (s.qItems < nA * nA) s.qItems = nA * nA;
  s.st = o; o += 4 * s.qItems;
  // chunk point: w, ex, visited, then type-2 U[l], r^k, Ka, Kb or type-1 U, r^k, K
  s.ckStride = 3 + nE + nA + 2 * (LB + nE);
  if (s.ckStride < 4 + 2 * nA) s.ckStride = 4 + 2 * nA;
  s.ck = o; o += (2 * kChunkPairs + 1) * s.ckStride;
  s.total = o;
  return s;
}

// Records a timing event; under stream capture as an event-record node of
// the graph (a plain record there only orders the capture).
inline void record_timing(cudaEvent_t e, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  if (cs == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
  else cudaEventRecord(e, st);
}

// Device-side consumers (ecp_grad.cu): the gradient contraction of an
// order-1 job's blocks with a density matrix (added to grad[3 * nAtoms]), and
// the energy of the upper-triangle AO matrix V.
void launch_gradient(const DevJob &J, const double *D, int ldD, double *grad, cudaStream_t st);
void launch_energy(const double *V, int dim, const double *D, int ldD, double *E, cudaStream_t st);
// Both blocks of every emitted unit in real spherical harmonics (sphOff per
// pair entry within a centre, sphStride values per centre).
void launch_to_sph(const DevJob &J, const double *c2s, const long long *sphOff, long long sphStride,
                   double *sout, cudaStream_t st);

// Launchers return 0, 3 when the shared memory does not fit, or
// kLaunchErrorBase + the cudaError_t of a failed launch.
constexpr int kLaunchErrorBase = 1000;

// Host-side launchers (ecp_fp64.cu).
int upload_schedules(const int *s93slot, int s93n, const int *s93lvEnd, const int *s93lvJ,
                     const int *s93lvN, int s93levels, const int *s92slot, int s92n,
                     const int *s92lvEnd, const int *s92lvN, int s92levels, void *stream);
// Launches the six-kernel pipeline on `stream`; u0/u1 (may be null) are
// recorded around the per-unit kernel.
int launch_fp64_pipeline(const DevJob &job, cudaStream_t stream, size_t smemBytes, cudaEvent_t u0,
                         cudaEvent_t u1);
// The four per-job kernels before the unit kernel (radii, centre potentials,
// centre-atom angular tables, windows + F tables) and the AO scatter after it.
void launch_prologue(const DevJob &job, cudaStream_t stream, bool withF);
void launch_epilogue(const DevJob &job, cudaStream_t stream);

// Batched path (ecp_fast.cu): same prologue/epilogue, warp-per-primitive-pair
// unit kernel with level-granular tabulation, Horner-form Bessel rows and a
// table-driven exp.  Its level schedules are this unit's own __constant__
// copies.
int upload_schedules_fast(const int *s93slot, int s93n, const int *s93lvEnd, const int *s93lvJ,
                          const int *s93lvN, int s93levels, const int *s92slot, int s92n,
                          const int *s92lvEnd, const int *s92lvN, int s92levels, void *stream);
size_t fast_smem_bytes(int LB, int LE, int gcap, int maxNP);
// CTAs of the batched unit kernel resident per SM at smemBytes.
int fast_ctas_per_sm(size_t smemBytes, int queue);
// Sets the batched kernels' function attributes on the current device (call
// before any graph capture).
void fast_prepare();
// Resets the per-run words (warning word, queue head).
void launch_reset(const DevJob &job, cudaStream_t stream);
int launch_fast_pipeline(const DevJob &job, cudaStream_t stream, size_t smemBytes, const FastConfig &cfg,
                         cudaEvent_t u0, cudaEvent_t u1);

}  // namespace ecpgb

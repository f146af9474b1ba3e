// ecp_noalloc.cu -- getIntegrals for callers that cannot allocate device memory.
//
// Some host programs own all GPU memory themselves: a quantum-chemistry code
// that hands the whole device to its own memory pool or arena, or a serving
// loop that must not pay for (or risk failing) an allocation in the middle of
// a request.  Such callers cannot let a library call cudaMalloc.  This entry
// point runs the same six FP64 kernels as getIntegrals, but every device
// buffer -- the packed inputs, the tables, the per-centre and per-unit work
// arrays, the result matrix -- is carved out of one file-scope device array
// of fixed size (kScratchBytes below).  That array exists on every GPU that
// loads the library and stays allocated until the process exits.
//
// Rules of use:
//   * Every call looks up the array's device address with
//     cudaGetSymbolAddress on the current device (the lookup allocates
//     nothing; looking it up each time keeps the address valid after a
//     cudaDeviceReset reloads the module).  The first call on a device also
//     loads the module there; make that first call before any stream capture
//     on the device.
//   * Every call shares the one array and overwrites it.  Inside the library
//     the engine lock is held from the first write into the array to the
//     final synchronisation, so two host threads calling this entry point do
//     not interleave their jobs; but calls that overlap on the GPU with other
//     work that reads or writes the array (a kernel of the caller's own that
//     was handed the array, or a copy queued on another stream) race.  Each
//     call synchronises the default stream before it returns.
//   * Jobs whose buffers do not fit are rejected with an error naming the
//     bytes needed; nothing is allocated to make them fit.
//   * No CUDA allocation of any kind happens here (no cudaMalloc / cudaFree /
//     cudaMallocHost / stream or event creation); host-side parsing uses the
//     ordinary C++ heap.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "ecp_engine.h"
#include "ecp_host.h"
#include "ecp_tables.h"
#include "libecp_gb300.h"

namespace ecpgb {

constexpr size_t kScratchBytes = 64ull << 20;  // 64 MiB per device
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of the scratch array on the current device.
static int scratch_address(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    set_error("no usable CUDA device for the no-allocation entry point");
    return 1;
  }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess || !p) {
    set_error("cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
    return 1;
  }
  *out = p;
  return 0;
}

// Bump allocator over the scratch array (256-byte aligned pieces).
struct Carver {
  char *base;
  size_t used = 0;
  template <class T>
  T *take(size_t n) {
    size_t off = (used + 255) & ~(size_t)255;
    used = off + (n ? n : 1) * sizeof(T);
    return (T *)(base + off);
  }
};

template <class T>
static bool put(T *dst, const std::vector<T> &v) {
  return v.empty() || cudaMemcpy(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

int run_matrix_noalloc(const ecpgb_system &s, int rowdim, double *I) {
  std::unique_lock<std::mutex> lk(engine_mutex());
  Parsed P;
  if (parse_system(s, P)) return 1;
  if (rowdim < P.dim) { set_error("rowdim %d < basis dimension %d", rowdim, P.dim); return 1; }
  if (P.deriv) { set_error("the AO matrix exists for derivative order 0 only"); return 1; }
  if (P.nCentres == 0 || P.nPairs == 0) return 0;
  HostTables h;
  build_tables(table_key(P), h);
  if (h.status) {
    set_error(h.status == 1 ? "Bessel series did not converge" : "table sizes out of range");
    return 1;
  }
  // The level schedules live in __constant__ memory shared with the engine
  // and with requests in flight on the server's streams: wait for those to
  // finish (the wait releases the lock) and upload this job's schedules
  // before the first write into the scratch array.  From here to the final
  // synchronisation the lock stays held, so no other call of this entry
  // point can rewrite the array under this job.
  wait_schedules_unpinned(lk);
  if (upload_schedules(h.s93.slot.data(), (int)h.s93.slot.size(), h.s93.lvEnd.data(), h.s93.lvJ.data(),
                       h.s93.lvN.data(), h.s93.nLevels, h.s92.slot.data(), (int)h.s92.slot.size(),
                       h.s92.lvEnd.data(), h.s92.lvN.data(), h.s92.nLevels, nullptr)) {
    set_error("schedule upload failed");
    return 1;
  }
  schedules_overwritten();
  void *sp = nullptr;
  if (scratch_address(&sp)) return 1;
  // used-triple lists per (la, lb, l), as the engine builds them
  const int LB = h.maxLBS, LE = h.maxLECP > 0 ? h.maxLECP : 1;
  std::vector<int> off, cnt, items, tmp;
  int nItemsMax = 0;
  for (int la = 0; la <= LB; la++)
    for (int lb = 0; lb <= LB; lb++) {
      int tot = 0;
      for (int l = 0; l < LE; l++) {
        used_triples(la, lb, l, tmp);
        off.push_back((int)items.size());
        cnt.push_back((int)tmp.size());
        items.insert(items.end(), tmp.begin(), tmp.end());
        tot += (int)tmp.size();
      }
      nItemsMax = tot > nItemsMax ? tot : nItemsMax;
    }
  if (nItemsMax > 2048) { set_error("angular momenta too high for the FP64 kernel"); return 1; }

  DevJob J;
  std::memset(&J, 0, sizeof J);
  J.nAtoms = P.nAtoms; J.nShells = P.nShells; J.nPrims = P.nPrims; J.nCentres = P.nCentres;
  J.nPairs = P.nPairs; J.dim = P.dim;
  J.maxLECP = h.maxLECP; J.maxLBS = h.maxLBS; J.maxLambda = h.maxLambda; J.nk = h.nk; J.nF = h.nF;
  J.tmDim = h.tmDim; J.tabL = h.tabL; J.besselN = h.besselN; J.omD1 = h.omD1; J.omD2 = h.omD2;
  J.angLam = h.maxLECP + h.maxLBS + 1;
  J.angLM = LE * LE;
  J.angC = ncum(h.maxLBS);
  J.uspD = h.maxLBS + 1;
  J.largeOrder = (int)h.xl.size();
  J.tol = P.tol; J.acc = P.acc;
  J.lnAcc1 = std::log(P.acc) - 2;
  J.lnAcc2 = std::log(1.0E-14) - 2;
  J.centreStride = P.centreStride;

  // carve every buffer; check the total before any copy
  Carver cv{(char *)sp};
  const size_t nc = P.nCentres, ns = P.nShells, na = P.nAtoms, O = kSmallOrder;
  double *geom = cv.take<double>(P.geom.size()), *pA = cv.take<double>(P.primA.size()),
         *pD = cv.take<double>(P.primD.size()), *tN = cv.take<double>(P.termN.size()),
         *tD = cv.take<double>(P.termD.size()), *tA = cv.take<double>(P.termA.size());
  int *shL = cv.take<int>(P.shL.size()), *shK = cv.take<int>(P.shK.size()), *shP = cv.take<int>(P.shP.size()),
      *shA = cv.take<int>(P.shAtom.size()), *shO = cv.take<int>(P.shAO.size()),
      *aM = cv.take<int>(P.atomMaxL.size()), *cA = cv.take<int>(P.ctrAtom.size()),
      *cL = cv.take<int>(P.ctrL.size()), *cT = cv.take<int>(P.ctrT0.size()),
      *cN = cv.take<int>(P.ctrNT.size()), *tL = cv.take<int>(P.termL.size()),
      *prA = cv.take<int>(P.pairA.size()), *prB = cv.take<int>(P.pairB.size());
  long long *pO = cv.take<long long>(P.pairOff.size());
  double *xs = cv.take<double>(h.xs.size()), *ws = cv.take<double>(h.ws.size()),
         *xl = cv.take<double>(h.xl.size()), *wl = cv.take<double>(h.wl.size()),
         *bT = cv.take<double>(h.besselT.size()), *bC = cv.take<double>(h.besselC.size()),
         *p2s = cv.take<double>(h.poly2sph.size()), *fac = cv.take<double>(h.fac.size()),
         *dfac = cv.take<double>(h.dfac.size()), *om = cv.take<double>(h.omega.size());
  int *ijk = cv.take<int>(h.ijk.size()), *ijkI = cv.take<int>(h.ijkIndex.size()),
      *iO = cv.take<int>(off.size()), *iC = cv.take<int>(cnt.size()), *iI = cv.take<int>(items.size());
  J.radius = cv.take<double>(ns);
  J.utab = cv.take<double>(nc * O * LE * h.nk);
  J.uL = cv.take<double>(nc * O);
  J.gridEnd = cv.take<int>(nc);
  J.win = cv.take<int>(nc * ns * 3);
  J.F = cv.take<double>(nc * ns * O * h.nF);
  J.cgeo = cv.take<double>(nc * na * 4);
  J.usp = cv.take<double>(nc * na * J.uspD * J.uspD * J.uspD);
  J.ang = cv.take<double>(nc * na * (size_t)J.angLam * J.angLM * J.angC);
  J.out = cv.take<double>(nc * (size_t)P.centreStride);
  J.status = cv.take<int>(nc * (size_t)P.nPairs);
  J.mat = cv.take<double>((size_t)P.dim * P.dim);
  J.errWord = cv.take<int>(2);
  if (cv.used > kScratchBytes) {
    set_error("job needs %zu bytes of device scratch; the no-allocation entry point has %zu",
              cv.used, kScratchBytes);
    return 1;
  }

  bool ok = put(geom, P.geom) && put(pA, P.primA) && put(pD, P.primD) && put(tN, P.termN) &&
            put(tD, P.termD) && put(tA, P.termA) && put(shL, P.shL) && put(shK, P.shK) &&
            put(shP, P.shP) && put(shA, P.shAtom) && put(shO, P.shAO) && put(aM, P.atomMaxL) &&
            put(cA, P.ctrAtom) && put(cL, P.ctrL) && put(cT, P.ctrT0) && put(cN, P.ctrNT) &&
            put(tL, P.termL) && put(prA, P.pairA) && put(prB, P.pairB) && put(pO, P.pairOff) &&
            put(xs, h.xs) && put(ws, h.ws) && put(xl, h.xl) && put(wl, h.wl) && put(bT, h.besselT) &&
            put(bC, h.besselC) && put(p2s, h.poly2sph) && put(fac, h.fac) && put(dfac, h.dfac) &&
            put(om, h.omega) && put(ijk, h.ijk) && put(ijkI, h.ijkIndex) && put(iO, off) &&
            put(iC, cnt) && put(iI, items);
  // the matrix starts as the caller's I (this call adds to it, like getIntegrals);
  // the error words start at "no warning"
  const int init[2] = {INT_MAX, 0};
  ok = ok && cudaMemcpy2D(J.mat, sizeof(double) * P.dim, I, sizeof(double) * rowdim,
                          sizeof(double) * P.dim, P.dim, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(J.errWord, init, sizeof init, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) { set_error("copy into the scratch array failed"); return 1; }
  J.geom = geom; J.primA = pA; J.primD = pD; J.termN = tN; J.termD = tD; J.termA = tA;
  J.shL = shL; J.shK = shK; J.shP = shP; J.shAtom = shA; J.shAO = shO; J.atomMaxL = aM;
  J.ctrAtom = cA; J.ctrL = cL; J.ctrT0 = cT; J.ctrNT = cN; J.termL = tL;
  J.pairA = prA; J.pairB = prB; J.pairOff = pO;
  J.xSmall = xs; J.wSmall = ws; J.xLarge = xl; J.wLarge = wl; J.besT = bT; J.besC = bC;
  J.p2s = p2s; J.fac = fac; J.dfac = dfac; J.omega = om; J.ijk = ijk; J.ijkIdx = ijkI;
  J.itemOff = iO; J.itemCnt = iC; J.items = iI;

  UnitSmem Lm = unit_smem_layout(h.maxLBS, h.maxLECP, h.nF);
  if (launch_fp64_pipeline(J, nullptr, sizeof(double) * (size_t)Lm.total, nullptr, nullptr)) {
    set_error("kernel launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    return 1;
  }
  int err[2] = {0, 0};
  ok = cudaMemcpy2D(I, sizeof(double) * rowdim, J.mat, sizeof(double) * P.dim, sizeof(double) * P.dim,
                    P.dim, cudaMemcpyDeviceToHost) == cudaSuccess &&
       cudaMemcpy(err, J.errWord, sizeof err, cudaMemcpyDeviceToHost) == cudaSuccess &&
       cudaStreamSynchronize(nullptr) == cudaSuccess;
  if (!ok) { set_error("device error: %s", cudaGetErrorString(cudaGetLastError())); return 1; }
  if (err[1]) { set_error("a shell radius did not converge (Newton, 40 steps)"); return 1; }
  return err[0] == INT_MAX ? 0 : 2;
}

}  // namespace ecpgb

extern "C" int ecpgb_getIntegrals_noalloc(const ecpgb_system *s, int rowdim, double *I) {
  if (!s || !I) {
    ecpgb::set_error("null system or matrix");
    return 1;
  }
  return ecpgb::run_matrix_noalloc(*s, rowdim, I);
}

extern "C" long long ecpgb_noalloc_capacity(void) { return (long long)ecpgb::kScratchBytes; }

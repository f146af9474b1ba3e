// ecp_host.cu -- host side of the engine: parsing, resident tables, device
// buffers, the run sequence, the device-resident job and the pipe probe.
//
// One run of a job on the engine's stream:
//   one H2D copy of all inputs (packed into a pinned staging buffer), memsets
//   of the AO matrix / block buffer / error words, the six-kernel FP64
//   pipeline, one D2H copy of the result (matrix or blocks) and the error
//   words.  Tables (grids, Bessel table, angular table, ...) are built once
//   per key on the host and stay resident on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "ecp_engine.h"
#include "ecp_host.h"
#include "ecp_tables.h"

namespace ecpgb {

static thread_local std::string g_err;
const char *last_error() { return g_err.c_str(); }
void set_error(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
}

#define CUDA_OK(x)                                                                   \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      set_error("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return -1;                                                                     \
    }                                                                                \
  } while (0)

// ------------------------------------------------------------------ parsing

static const int kShiftA[3][10] = {{0}, {+1, -1, 0, 0}, {+2, -2, +1, +1, -1, -1, 0, 0, +1, 0}};
static const int kShiftB[3][10] = {{0}, {0, 0, +1, -1}, {0, 0, +1, -1, +1, -1, +2, -2, 0, +1}};

int shift_count(int deriv) { return deriv == 0 ? 1 : deriv == 1 ? 4 : 10; }

void shift_pair(int deriv, int s, int &shifta, int &shiftb) {
  shifta = kShiftA[deriv][s];
  shiftb = kShiftB[deriv][s];
}

// The derivative scheme sizes every table for basis l up to maxLBS + n
// (src/libecp.c:144-147): the tables of a job whose largest shell is shifted.
TableKey table_key(const Parsed &P) {
  return {P.maxLECP, P.maxLBS + P.deriv, P.largeGridOrder, P.tol, P.acc, P.ordering};
}

void shift_block_l(int deriv, int la, int lb, int shifta, int shiftb, int &lpa, int &lpb) {
  lpa = la + shifta;
  lpb = lb + shiftb;
  if (deriv == 2) {
    if (shifta == 1 && shiftb == 0) lpa = la;
    else if (shifta == 0 && shiftb == 1) lpb = lb;
  }
}

int parse_system(const ecpgb_system &s, Parsed &P) {
  P = Parsed();
  if (s.nrAtoms < 1 || !s.geometry || !s.shellsECP || !s.shellsBS) {
    set_error("invalid system: nrAtoms < 1 or missing arrays");
    return 1;
  }
  P.nAtoms = s.nrAtoms;
  P.geom.assign(s.geometry, s.geometry + 3 * s.nrAtoms);
  P.atomMaxL.assign(s.nrAtoms, 0);
  P.atomShell0.assign(s.nrAtoms, 0);
  int sh = 0, prim = 0, ao = 0;
  for (int a = 0; a < s.nrAtoms; a++) {
    P.atomShell0[a] = sh;
    if (s.shellsBS[a] < 0) { set_error("negative shell count on atom %d", a); return 1; }
    for (int j = 0; j < s.shellsBS[a]; j++, sh++) {
      int l = s.lBS[sh], k = s.KBS[sh];
      if (l < 0 || l > kMaxLBasis) { set_error("basis l=%d outside 0..%d", l, kMaxLBasis); return 1; }
      if (k < 1 || k > kMaxContraction) {
        set_error("contraction %d outside 1..%d", k, kMaxContraction);
        return 1;
      }
      P.shL.push_back(l); P.shK.push_back(k); P.shP.push_back(prim); P.shAtom.push_back(a);
      P.shAO.push_back(ao); P.shLocal.push_back(j);
      for (int p = 0; p < k; p++) { P.primA.push_back(s.aBS[prim + p]); P.primD.push_back(s.dBS[prim + p]); }
      prim += k;
      ao += ncart(l);
      P.atomMaxL[a] = std::max(P.atomMaxL[a], l);
      P.maxLBS = std::max(P.maxLBS, l);
    }
  }
  P.nShells = sh;
  P.nPrims = prim;
  P.dim = ao;
  // ECPs (src/libecp.c:93-127): per atom its shells' terms in order
  int esh = 0, term = 0;
  for (int a = 0; a < s.nrAtoms; a++) {
    if (s.shellsECP[a] <= 0) {
      esh += 0;
      continue;
    }
    int L = 0, t0 = (int)P.termL.size();
    for (int j = 0; j < s.shellsECP[a]; j++, esh++) {
      int l = s.lECP[esh], k = s.KECP[esh];
      if (l < 0 || l > kMaxLEcp || k < 0) {
        set_error("ECP shell with l=%d (0..%d) or K=%d", l, kMaxLEcp, k);
        return 1;
      }
      L = std::max(L, l);
      for (int t = 0; t < k; t++, term++) {
        P.termL.push_back(l);
        P.termN.push_back(s.nECP[term]);
        P.termD.push_back(s.dECP[term]);
        P.termA.push_back(s.aECP[term]);
      }
    }
    P.ctrAtom.push_back(a);
    P.ctrL.push_back(L);
    P.ctrT0.push_back(t0);
    P.ctrNT.push_back((int)P.termL.size() - t0);
    P.maxLECP = std::max(P.maxLECP, L);
  }
  P.nCentres = (int)P.ctrAtom.size();
  if (s.derivative < 0 || s.derivative > 2) {
    set_error("derivative order %d outside 0..2", s.derivative);
    return 1;
  }
  P.deriv = s.derivative;
  P.nShift = shift_count(P.deriv);
  if (s.shellOrdering) {
    // src/libecp.c:159: the order must reach maxLambda + maxAlpha + 1
    const int need = P.maxLECP + 2 * (P.maxLBS + P.deriv);
    if (s.orderingLmax < need) {
      set_error("shellOrdering covers l <= %d; this job needs l <= %d", s.orderingLmax, need);
      return 1;
    }
    const int lmax = s.orderingLmax;
    if (lmax > 24) { set_error("orderingLmax %d too large", lmax); return 1; }
    P.ordering.assign(s.shellOrdering, s.shellOrdering + 3 * ncum(lmax));
    for (int l = 0; l <= lmax; l++) {  // each shell a permutation of its exponent triples
      std::vector<char> seen((size_t)(l + 1) * (l + 1), 0);
      for (int c = 0; c < ncart(l); c++) {
        const int *e = &P.ordering[3 * (ncum(l - 1) + c)];
        if (e[0] < 0 || e[1] < 0 || e[2] < 0 || e[0] + e[1] + e[2] != l || seen[e[0] * (l + 1) + e[1]]) {
          set_error("shellOrdering: shell l = %d is not an order of its Cartesian functions", l);
          return 1;
        }
        seen[e[0] * (l + 1) + e[1]] = 1;
      }
    }
  }
  if (P.maxLBS + P.deriv > kMaxLBasis) {  // the shifted shells must fit the tables
    set_error("basis l %d with derivative order %d: shifted l above %d", P.maxLBS, P.deriv, kMaxLBasis);
    return 1;
  }
  // shell pairs in the reference's loop order (src/libecp.c:278-312), each
  // with its derivative shifts innermost (src/libecp.c:322); a shift that
  // lowers l below 0 has no blocks
  long long off = 0;
  for (int A = 0; A < s.nrAtoms; A++)
    for (int B = A; B < s.nrAtoms; B++)
      for (int i = 0; i < s.shellsBS[A]; i++)
        for (int j = 0; j < s.shellsBS[B]; j++) {
          if (A == B && j < i) continue;
          int sa = P.atomShell0[A] + i, sb = P.atomShell0[B] + j;
          for (int k = 0; k < P.nShift; k++) {
            int ha, hb, lpa, lpb;
            shift_pair(P.deriv, k, ha, hb);
            P.pairA.push_back(sa);
            P.pairB.push_back(sb);
            P.pairShift.push_back(k);
            P.pairOff.push_back(off);
            if (P.shL[sa] + ha < 0 || P.shL[sb] + hb < 0) continue;
            shift_block_l(P.deriv, P.shL[sa], P.shL[sb], ha, hb, lpa, lpb);
            off += 2LL * ncart(lpa) * ncart(lpb);
          }
        }
  P.nPairs = (int)P.pairA.size();
  P.centreStride = off;
  P.largeGridOrder = s.largeGridOrder;
  P.tol = s.tolerance;
  P.acc = s.accuracy;
  // the grid has 2^floor(log2(order + 1)) - 1 points: at most kMaxLargeOrder
  // up to order 2 (kMaxLargeOrder + 1) - 2
  if (s.largeGridOrder < 384 || s.largeGridOrder > 2 * (kMaxLargeOrder + 1) - 2) {
    set_error("largeGridOrder %d outside 384..%d", s.largeGridOrder, 2 * (kMaxLargeOrder + 1) - 2);
    return 1;
  }
  if (!(s.accuracy > 0) || !(s.tolerance > 0)) {
    set_error("tolerance and accuracy must be positive");
    return 1;
  }
  return 0;
}

// ------------------------------------------------------------ device tables

struct DevTables {
  TableKey key{};
  HostTables host;
  DBuf<float> besHf, besAf, besZf, xlf, wlf;  // float pairs (mixed path)
  DBuf<double> xs, ws, xl, wl, besT, besC, besH, besA, besZ, shNorm, p2s, fac, dfac, omega, c2s;
  DBuf<int> ijk, ijkIdx, itemOff, itemCnt, items, s93, s92;
  DBuf<short> byN93;
  int nItemsMax = 0;
};

// The small-grid schedule's slots step by step (33, then 32 at a time) in
// ascending order of their grid point (the batched kernel's type-1 steps).
static std::vector<short> by_point_order(const std::vector<int> &slot) {
  const int n = (int)slot.size();
  std::vector<short> out(n);
  for (int s0 = 0; s0 < n;) {
    int s1 = s0 == 0 ? 33 : s0 + 32;
    if (s1 > n) s1 = n;
    for (int t = s0; t < s1; t++) out[t] = (short)t;
    std::sort(out.begin() + s0, out.begin() + s1, [&](short a, short b) { return slot[a] < slot[b]; });
    s0 = s1;
  }
  return out;
}

// Two table sets share level schedules when their grids are the same.
static bool same_schedules(const DevTables *a, const DevTables *b) {
  return a->host.s93.slot == b->host.s93.slot && a->host.s92.slot == b->host.s92.slot &&
         a->host.s93.lvEnd == b->host.s93.lvEnd && a->host.s92.lvEnd == b->host.s92.lvEnd;
}

struct Engine {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  // timing events of the one-shot runs (matrix, blocks), created once
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // batched-path launch configuration per (maxLBS, maxLECP), set by the autotuner
  std::map<std::pair<int, int>, FastConfig> tuned;
  FastConfig config_for(int LB, int LE) const {
    auto it = tuned.find({LB, LE});
    return it == tuned.end() ? FastConfig{} : it->second;
  }
  std::vector<std::unique_ptr<DevTables>> tables;
  const DevTables *schedOwner = nullptr;
  JobBuffers shared;
  DBuf<char> flush;
  DBuf<unsigned long long> classCycles;  // autotuner: per-class cycle counts
  DBuf<double> dens, gradBuf;  // density matrix and gradient of run_gradient
  bool init = false;

  int ensure_init() {
    if (init) return 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) {
      set_error("no CUDA device: the ECP engine runs on the GPU only");
      return -1;
    }
    CUDA_OK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (auto &e : ev) CUDA_OK(cudaEventCreate(&e));
    init = true;
    return 0;
  }

  const DevTables *get_tables(const TableKey &key) {
    for (auto &t : tables)
      if (t->key == key) return t.get();
    if (tables.size() >= 256) {
      set_error("more than 256 distinct table keys (ECP L, basis l, grid order, accuracy)");
      return nullptr;
    }
    auto t = std::make_unique<DevTables>();
    t->key = key;
    build_tables(key, t->host);
    if (t->host.status) {
      set_error(t->host.status == 1 ? "Bessel series did not converge" : "table sizes out of range");
      return nullptr;
    }
    HostTables &h = t->host;
    bool ok = t->xs.upload(h.xs, stream) && t->ws.upload(h.ws, stream) && t->xl.upload(h.xl, stream) &&
              t->wl.upload(h.wl, stream) && t->besT.upload(h.besselT, stream) &&
              t->besC.upload(h.besselC, stream) && t->p2s.upload(h.poly2sph, stream) &&
              t->fac.upload(h.fac, stream) && t->dfac.upload(h.dfac, stream) &&
              t->omega.upload(h.omega, stream) && t->ijk.upload(h.ijk, stream) &&
              t->ijkIdx.upload(h.ijkIndex, stream) && t->besH.upload(h.besselH, stream) && t->besA.upload(h.besselA, stream) && t->besHf.upload(h.besselHf, stream) &&
              t->besAf.upload(h.besselAf, stream) && t->besZf.upload(h.besselZf, stream) &&
              t->xlf.upload(h.xlf, stream) && t->wlf.upload(h.wlf, stream) &&
              t->besZ.upload(h.besselZ, stream) &&
              t->c2s.upload(h.cart2sph, stream) && t->s93.upload(h.s93.slot, stream) &&
              t->s92.upload(h.s92.slot, stream) && t->byN93.upload(by_point_order(h.s93.slot), stream) &&
              t->shNorm.upload(h.shNorm, stream);
    // used-triple lists per (la, lb, l)
    int LB = h.maxLBS, LE = h.maxLECP > 0 ? h.maxLECP : 1;
    std::vector<int> off, cnt, items, tmp;
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
        t->nItemsMax = std::max(t->nItemsMax, tot);
      }
    ok = ok && t->itemOff.upload(off, stream) && t->itemCnt.upload(cnt, stream) &&
         t->items.upload(items, stream);
    if (!ok) {
      set_error("device allocation failed for tables");
      return nullptr;
    }
    if (t->nItemsMax > 2048) {
      set_error("angular momenta too high for the FP64 kernel (%d radial items)", t->nItemsMax);
      return nullptr;
    }
    // tables live as long as the process: resident jobs and requests in
    // flight hold pointers to them
    tables.push_back(std::move(t));
    return tables.back().get();
  }

  // Requests in flight on the server's streams pin the current schedules;
  // a caller that needs other schedules waits (lock held by the caller,
  // passed in so the wait can release it) until no pin is left.
  int schedPins = 0;
  std::condition_variable cv;

  int use_schedules(const DevTables *t, std::unique_lock<std::mutex> *lk = nullptr) {
    if (schedOwner == t) return 0;
    if (schedOwner && same_schedules(schedOwner, t)) {
      schedOwner = t;
      return 0;
    }
    if (schedPins > 0) {
      if (!lk) {
        set_error("level schedules are pinned by requests in flight");
        return -1;
      }
      cv.wait(*lk, [&] { return schedPins == 0; });
      if (schedOwner == t) return 0;
    }
    const HostTables &h = t->host;
    int rc = upload_schedules(h.s93.slot.data(), (int)h.s93.slot.size(), h.s93.lvEnd.data(),
                              h.s93.lvJ.data(), h.s93.lvN.data(), h.s93.nLevels, h.s92.slot.data(),
                              (int)h.s92.slot.size(), h.s92.lvEnd.data(), h.s92.lvN.data(),
                              h.s92.nLevels, stream);
    if (!rc)
      rc = upload_schedules_fast(h.s93.slot.data(), (int)h.s93.slot.size(), h.s93.lvEnd.data(),
                                 h.s93.lvJ.data(), h.s93.lvN.data(), h.s93.nLevels, h.s92.slot.data(),
                                 (int)h.s92.slot.size(), h.s92.lvEnd.data(), h.s92.lvN.data(),
                                 h.s92.nLevels, stream);
    if (rc) {
      set_error("schedule upload failed (%d)", rc);
      return -1;
    }
    schedOwner = t;
    return 0;
  }
};

static Engine &engine() {
  static Engine *e = new Engine();  // lives until exit; device memory is released by the driver
  return *e;
}

std::mutex &engine_mutex() { return engine().mu; }
void schedules_overwritten() { engine().schedOwner = nullptr; }
int engine_pin_request(const Parsed &P, const DevTables **T) {
  Engine &E = engine();
  if (E.ensure_init()) return 1;
  const DevTables *t = E.get_tables(table_key(P));
  if (!t) return 1;
  if (E.schedPins > 0 && E.schedOwner != t && !(E.schedOwner && same_schedules(E.schedOwner, t))) return 4;
  if (E.use_schedules(t)) return 1;
  E.schedPins++;
  *T = t;
  return 0;
}

void engine_unpin_request() {
  Engine &E = engine();
  if (E.schedPins > 0 && --E.schedPins == 0) E.cv.notify_all();
}

void wait_schedules_unpinned(std::unique_lock<std::mutex> &lk) {
  Engine &E = engine();
  E.cv.wait(lk, [&] { return E.schedPins == 0; });
}

// ------------------------------------------------------------ job set-up

static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

cudaStream_t &alloc_stream() {
  static thread_local cudaStream_t s = nullptr;
  return s;
}

static std::mutex g_retiredMu;
std::vector<void *> &retired_pinned() {
  static std::vector<void *> v;
  return v;
}
void retire_pinned(void *p) {
  std::lock_guard<std::mutex> lk(g_retiredMu);
  retired_pinned().push_back(p);
}
void free_retired_pinned() {
  std::lock_guard<std::mutex> lk(g_retiredMu);
  for (void *p : retired_pinned()) cudaFreeHost(p);
  retired_pinned().clear();
}

bool valid_mode(int mode) { return mode == ECPGB_FP64 || mode == ECPGB_FAST || mode == ECPGB_MIXED; }

// The class-major work queue: units grouped by their (la, lb, L) class --
// largest la + lb first, then la, then the centre's L descending -- and
// within a class by descending estimated cost, ties in the reference's order.
// Concurrent CTAs then mostly run units of one class, i.e. the same code
// paths and table widths.  Empty when the units do not fit 31-bit indices.
static void unit_order_class(const Parsed &P, std::vector<int> &order) {
  order.clear();
  const long long n = (long long)P.nCentres * P.nPairs;
  if (n <= 0 || n >= INT_MAX) return;
  // two stable counting sorts (least significant key first): by descending
  // cost, then by class
  std::vector<int> pc(P.nPairs), cc(P.nCentres), pcls(P.nPairs);
  int maxP = 0, maxC = 0, LB = 0, LE = 0;
  for (int c = 0; c < P.nCentres; c++) { cc[c] = P.ctrL[c] + 2; maxC = std::max(maxC, cc[c]); LE = std::max(LE, P.ctrL[c]); }
  for (int p = 0; p < P.nPairs; p++) {
    const int a = P.pairA[p], b = P.pairB[p];
    pc[p] = P.shK[a] * P.shK[b] * (P.shL[a] + P.shL[b] + 2);
    maxP = std::max(maxP, pc[p]);
    LB = std::max(LB, std::max(P.shL[a], P.shL[b]));
  }
  const long long nCost = (long long)maxP * maxC + 1;
  if (nCost > (1 << 24)) return;
  const int W1 = LB + 1, W2 = LE + 1, nCls = (2 * LB + 1) * W1 * W2;
  for (int p = 0; p < P.nPairs; p++) {
    const int la = P.shL[P.pairA[p]], lb = P.shL[P.pairB[p]];
    pcls[p] = ((2 * LB - la - lb) * W1 + (LB - la)) * W2;  // + (LE - L) per centre
  }
  std::vector<int> tmp(n);
  std::vector<int> start(std::max<long long>(nCost, nCls) + 1);
  // pass 1: by descending cost, ties in the reference's order
  std::fill(start.begin(), start.begin() + nCost + 1, 0);
  for (int c = 0; c < P.nCentres; c++)
    for (int p = 0; p < P.nPairs; p++) start[nCost - 1 - (long long)pc[p] * cc[c]]++;
  for (long long k = 0, acc = 0; k <= nCost; k++) { const int v = start[k]; start[k] = (int)acc; acc += v; }
  for (int c = 0; c < P.nCentres; c++)
    for (int p = 0; p < P.nPairs; p++) tmp[start[nCost - 1 - (long long)pc[p] * cc[c]]++] = c * P.nPairs + p;
  // pass 2: by class, stable
  auto cls = [&](int u) { const int c = u / P.nPairs; return pcls[u % P.nPairs] + (LE - P.ctrL[c]); };
  std::fill(start.begin(), start.begin() + nCls + 1, 0);
  for (long long i = 0; i < n; i++) start[cls(tmp[i])]++;
  for (int k = 0, acc = 0; k <= nCls; k++) { const int v = start[k]; start[k] = acc; acc += v; }
  order.resize(n);
  for (long long i = 0; i < n; i++) order[start[cls(tmp[i])]++] = tmp[i];
}

// The work queue of the batched path: units by descending estimated cost,
// primitive pairs x (la + lb + 2) x (L + 2), ties in the reference's order
// (a stable counting sort).  Empty when the units do not fit 31-bit indices.
static void unit_order(const Parsed &P, std::vector<int> &order) {
  order.clear();
  const long long n = (long long)P.nCentres * P.nPairs;
  if (n <= 0 || n >= INT_MAX) return;
  std::vector<int> pk(P.nPairs), ck(P.nCentres);
  int maxP = 0, maxC = 0;
  for (int p = 0; p < P.nPairs; p++) {
    int a = P.pairA[p], b = P.pairB[p];
    pk[p] = P.shK[a] * P.shK[b] * (P.shL[a] + P.shL[b] + 2);
    maxP = std::max(maxP, pk[p]);
  }
  for (int c = 0; c < P.nCentres; c++) {
    ck[c] = P.ctrL[c] + 2;
    maxC = std::max(maxC, ck[c]);
  }
  const long long nk = (long long)maxP * maxC + 1;
  if (nk > (1 << 24)) return;
  std::vector<int> start(nk + 1, 0);
  for (int c = 0; c < P.nCentres; c++)
    for (int p = 0; p < P.nPairs; p++) start[nk - 1 - pk[p] * ck[c]]++;
  int acc = 0;
  for (long long k = 0; k <= nk; k++) {
    int v = start[k];
    start[k] = acc;
    acc += v;
  }
  order.resize(n);
  for (int c = 0; c < P.nCentres; c++)
    for (int p = 0; p < P.nPairs; p++) order[start[nk - 1 - pk[p] * ck[c]]++] = c * P.nPairs + p;
}

// Packs the inputs into the pinned staging buffer, copies them to the device
// and fills the DevJob's input and work pointers.
size_t job_device_bytes(const Parsed &P, int mode) {
  const size_t nc = P.nCentres, ns = P.nShells, na = P.nAtoms, O = kSmallOrder;
  const size_t LE = P.maxLECP > 0 ? P.maxLECP : 1, LB = P.maxLBS + P.deriv;
  const size_t nk = std::max(LB + LE, 2 * LB) + 1, nF = LB + LE + 1, D = LB + 1;  // table ranks (upper bounds)
  const size_t angLam = P.maxLECP + LB + 1, angC = (LB + 1) * (LB + 2) * (LB + 3) / 6;
  size_t in = 8 * (P.geom.size() + P.primA.size() + P.primD.size() + 3 * P.termL.size() + P.pairOff.size()) +
              4 * (5 * P.shL.size() + P.atomMaxL.size() + 4 * P.ctrAtom.size() + P.termL.size() + 3 * P.pairA.size()) +
              (mode != ECPGB_FP64 ? 8 * nc * P.nPairs : 0) + (mode == ECPGB_MIXED ? 16 * P.termL.size() : 0) +
              24 * 256;
  size_t work = 8 * (ns + nc * O * LE * nk + nc * O + nc * ns * (1 + P.deriv) * O * nF + nc * na * 4 + nc * na * D * D * D +
                     nc * na * angLam * LE * LE * angC + nc * (size_t)P.centreStride + (size_t)P.dim * P.dim) +
                4 * (nc + nc * ns * 3 + nc * (size_t)P.nPairs + 2) + 8;
  return in + work;
}

int stage_job(const Parsed &P, const DevTables *T, JobBuffers &B, DevJob &J, int mode, cudaStream_t stream) {
  const HostTables &h = T->host;
  std::memset(&J, 0, sizeof J);
  J.nAtoms = P.nAtoms; J.nShells = P.nShells; J.nPrims = P.nPrims; J.nCentres = P.nCentres;
  J.nPairs = P.nPairs; J.dim = P.dim;
  J.maxLECP = h.maxLECP; J.maxLBS = h.maxLBS; J.maxLambda = h.maxLambda; J.nk = h.nk; J.nF = h.nF;
  J.tmDim = h.tmDim; J.tabL = h.tabL; J.besselN = h.besselN; J.omD1 = h.omD1; J.omD2 = h.omD2;
  int LE = h.maxLECP > 0 ? h.maxLECP : 1;
  J.angLam = h.maxLECP + h.maxLBS + 1;
  J.angLM = LE * LE;
  J.angC = ncum(h.maxLBS);
  J.uspD = h.maxLBS + 1;
  J.largeOrder = (int)h.xl.size();
  for (int k : P.shK) J.maxNP = std::max(J.maxNP, k * k);
  J.tol = P.tol; J.acc = P.acc;
  J.lnAcc1 = std::log(P.acc) - 2;
  J.lnAcc2 = std::log(1.0E-14) - 2;
  // --- inputs: one packed H2D copy
  struct Piece { const void *src; size_t bytes; size_t off; };
  std::vector<Piece> pcs;
  size_t tot = 0;
  auto add = [&](const void *src, size_t bytes) {
    pcs.push_back({src, bytes, tot});
    tot += al(bytes ? bytes : 1);
    return pcs.size() - 1;
  };
  size_t iGeom = add(P.geom.data(), 8 * P.geom.size()), iPA = add(P.primA.data(), 8 * P.primA.size()),
         iPD = add(P.primD.data(), 8 * P.primD.size()), iTN = add(P.termN.data(), 8 * P.termN.size()),
         iTD = add(P.termD.data(), 8 * P.termD.size()), iTA = add(P.termA.data(), 8 * P.termA.size()),
         iShL = add(P.shL.data(), 4 * P.shL.size()), iShK = add(P.shK.data(), 4 * P.shK.size()),
         iShP = add(P.shP.data(), 4 * P.shP.size()), iShA = add(P.shAtom.data(), 4 * P.shAtom.size()),
         iShO = add(P.shAO.data(), 4 * P.shAO.size()), iAM = add(P.atomMaxL.data(), 4 * P.atomMaxL.size()),
         iCA = add(P.ctrAtom.data(), 4 * P.ctrAtom.size()), iCL = add(P.ctrL.data(), 4 * P.ctrL.size()),
         iCT = add(P.ctrT0.data(), 4 * P.ctrT0.size()), iCN = add(P.ctrNT.data(), 4 * P.ctrNT.size()),
         iTL = add(P.termL.data(), 4 * P.termL.size()), iPrA = add(P.pairA.data(), 4 * P.pairA.size()),
         iPrB = add(P.pairB.data(), 4 * P.pairB.size()), iPO = add(P.pairOff.data(), 8 * P.pairOff.size()),
         iPS = add(P.pairShift.data(), 4 * P.pairShift.size());
  std::vector<int> order, orderClass;
  if (mode != ECPGB_FP64) {
    unit_order(P, order);
    unit_order_class(P, orderClass);
  }
  size_t iOrd = add(order.data(), 4 * order.size()), iOrdC = add(orderClass.data(), 4 * orderClass.size());
  // the ECP terms' exponents and coefficients as float pairs (mixed path)
  std::vector<float> tAf, tDf;
  if (mode == ECPGB_MIXED) {
    split_pairs(P.termA, tAf);
    split_pairs(P.termD, tDf);
  }
  size_t iTAf = add(tAf.data(), 4 * tAf.size()), iTDf = add(tDf.data(), 4 * tDf.size());
  if (!B.pinned.ensure(tot) || !B.in.ensure(tot)) {
    set_error("allocation of %zu input bytes failed", tot);
    return -1;
  }
  for (auto &p : pcs)
    if (p.bytes) std::memcpy(B.pinned.p + p.off, p.src, p.bytes);
  CUDA_OK(cudaMemcpyAsync(B.in.p, B.pinned.p, tot, cudaMemcpyHostToDevice, stream));
  B.h2dBytes = (long long)tot;
  auto dp = [&](size_t i) { return (void *)(B.in.p + pcs[i].off); };
  J.geom = (const double *)dp(iGeom); J.primA = (const double *)dp(iPA); J.primD = (const double *)dp(iPD);
  J.termN = (const double *)dp(iTN); J.termD = (const double *)dp(iTD); J.termA = (const double *)dp(iTA);
  J.shL = (const int *)dp(iShL); J.shK = (const int *)dp(iShK); J.shP = (const int *)dp(iShP);
  J.shAtom = (const int *)dp(iShA); J.shAO = (const int *)dp(iShO); J.atomMaxL = (const int *)dp(iAM);
  J.ctrAtom = (const int *)dp(iCA); J.ctrL = (const int *)dp(iCL); J.ctrT0 = (const int *)dp(iCT);
  J.ctrNT = (const int *)dp(iCN); J.termL = (const int *)dp(iTL); J.pairA = (const int *)dp(iPrA);
  J.pairB = (const int *)dp(iPrB); J.pairOff = (const long long *)dp(iPO);
  J.pairShift = (const int *)dp(iPS);
  J.termAf = mode == ECPGB_MIXED ? (const ff *)dp(iTAf) : nullptr;
  J.termDf = mode == ECPGB_MIXED ? (const ff *)dp(iTDf) : nullptr;
  J.deriv = P.deriv;
  J.nRuns = 1 + P.deriv;
  J.order = order.empty() ? nullptr : (const int *)dp(iOrd);
  J.orderClass = orderClass.empty() ? nullptr : (const int *)dp(iOrdC);
  J.centreStride = P.centreStride;
  // --- tables
  J.itemOff = T->itemOff.p; J.itemCnt = T->itemCnt.p; J.items = T->items.p;
  J.xSmall = T->xs.p; J.wSmall = T->ws.p; J.xLarge = T->xl.p; J.wLarge = T->wl.p;
  J.besT = T->besT.p; J.besC = T->besC.p; J.p2s = T->p2s.p; J.fac = T->fac.p; J.dfac = T->dfac.p;
  J.ijk = T->ijk.p; J.ijkIdx = T->ijkIdx.p; J.omega = T->omega.p;
  // --- work arrays
  const size_t nc = P.nCentres, ns = P.nShells, na = P.nAtoms, O = kSmallOrder;
  bool ok = B.radius.ensure(ns + 1) && B.utab.ensure(nc * O * LE * h.nk + 1) && B.uL.ensure(nc * O + 1) &&
            B.gridEnd.ensure(nc + 1) && B.win.ensure(nc * ns * 3 + 1) && B.F.ensure(nc * ns * (1 + P.deriv) * O * h.nF + 1) &&
            B.cgeo.ensure(nc * na * 4 + 1) && B.usp.ensure(nc * na * J.uspD * J.uspD * J.uspD + 1) &&
            B.ang.ensure(nc * na * (size_t)J.angLam * J.angLM * J.angC + 1) &&
            B.out.ensure(nc * (size_t)P.centreStride + 1) && B.status.ensure(nc * (size_t)P.nPairs + 1) &&
            B.mat.ensure((size_t)P.dim * P.dim + 1) && B.err.ensure(2) && B.head.ensure(1);
  if (!ok) {
    set_error("device allocation failed for the job's work arrays");
    return -1;
  }
  J.radius = B.radius.p; J.utab = B.utab.p; J.uL = B.uL.p; J.gridEnd = B.gridEnd.p; J.win = B.win.p;
  J.F = B.F.p; J.cgeo = B.cgeo.p; J.usp = B.usp.p; J.ang = B.ang.p; J.out = B.out.p;
  J.status = B.status.p; J.mat = B.mat.p; J.errWord = B.err.p; J.queueHead = B.head.p;
  if (mode != ECPGB_FP64) {  // screening stage buffers of the batched path
    const size_t nu = nc * (size_t)P.nPairs;
    if (!B.live.ensure(nu + 1) || !B.screenBlocks.ensure(nu / 256 + 2) || !B.liveCount.ensure(1)) {
      set_error("device allocation failed for the screening stage");
      return -1;
    }
    J.live = B.live.p;
    J.liveCount = B.liveCount.p;
    J.screenBlocks = B.screenBlocks.p;
  }
  J.gcap = FastConfig{}.gcap;
  J.besH = T->besH.p;
  J.besA = T->besA.p;
  J.besZ = T->besZ.p;
  J.besHf = (const ff *)T->besHf.p;
  J.besAf = (const ff *)T->besAf.p;
  J.besZf = (const ff *)T->besZf.p;
  J.xLf = (const ff *)T->xlf.p;
  J.wLf = (const ff *)T->wlf.p;
  J.s93 = T->s93.p;
  J.s92 = T->s92.p;
  J.byN93 = T->byN93.p;
  J.mixed = mode == ECPGB_MIXED;
  J.besHL = h.besselHL;
  J.shNorm = T->shNorm.p;
  UnitSmem L = unit_smem_layout(h.maxLBS, h.maxLECP, h.nF);
  B.smem = sizeof(double) * (size_t)L.total;
  return 0;
}

// Resets the per-run outputs and launches the pipeline of the mode (the
// batched path with launch configuration cfg).
int run_pipeline(JobBuffers &B, const DevJob &J, int mode, cudaEvent_t u0, cudaEvent_t u1,
                 const FastConfig *cfg, cudaStream_t stream) {
  launch_reset(J, stream);
  CUDA_OK(cudaMemsetAsync(B.mat.p, 0, sizeof(double) * (size_t)J.dim * J.dim, stream));
  int rc;
  if (mode == ECPGB_FAST || mode == ECPGB_MIXED) {
    FastConfig c = cfg ? *cfg : engine().config_for(J.maxLBS, J.maxLECP);
    c.mixed = mode == ECPGB_MIXED;
    rc = launch_fast_pipeline(J, stream, fast_smem_bytes(J.maxLBS, J.maxLECP, c.gcap, J.maxNP), c, u0, u1);
  } else {
    rc = launch_fp64_pipeline(J, stream, B.smem, u0, u1);
  }
  if (rc) {
    if (rc >= kLaunchErrorBase) set_error("kernel launch failed: %s", cudaGetErrorString((cudaError_t)(rc - kLaunchErrorBase)));
    else set_error("kernel launch failed (%d)", rc);
    return -1;
  }
  return 0;
}

// ------------------------------------------------------------ public runs

int run_matrix(const ecpgb_system &s, int mode, int rowdim, double *I, ecpgb_info *info) {
  Engine &E = engine();
  std::unique_lock<std::mutex> lk(E.mu);
  if (!valid_mode(mode)) { set_error("unknown mode %d", mode); return 1; }
  if (E.ensure_init()) return 1;
  Parsed P;
  if (parse_system(s, P)) return 1;
  if (rowdim < P.dim) { set_error("rowdim %d < basis dimension %d", rowdim, P.dim); return 1; }
  if (P.deriv) { set_error("the AO matrix exists for derivative order 0 only (use the blocks)"); return 1; }
  if (P.nCentres == 0 || P.nPairs == 0) {
    if (info) { std::memset(info, 0, sizeof *info); info->firstFailed = -1; }
    return 0;
  }
  const DevTables *T = E.get_tables(table_key(P));
  if (!T || E.use_schedules(T, &lk)) return 1;
  JobBuffers &B = E.shared;
  DevJob J;
  if (stage_job(P, T, B, J, mode, E.stream)) return 1;
  cudaEvent_t e0 = E.ev[0], e1 = E.ev[1], u0 = E.ev[2], u1 = E.ev[3];
  cudaEventRecord(e0, E.stream);
  if (run_pipeline(B, J, mode, u0, u1, nullptr, E.stream)) return 1;
  cudaEventRecord(e1, E.stream);
  size_t mb = sizeof(double) * (size_t)P.dim * P.dim;
  if (!B.pinnedOut.ensure(mb)) { set_error("pinned allocation failed"); return 1; }
  cudaMemcpyAsync(B.pinnedOut.p, B.mat.p, mb, cudaMemcpyDeviceToHost, E.stream);
  cudaMemcpyAsync(B.pinnedErr, B.err.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, E.stream);
  cudaError_t ce = cudaStreamSynchronize(E.stream);
  if (ce != cudaSuccess) { set_error("device error: %s", cudaGetErrorString(ce)); return 1; }
  float ms = 0, msu = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventElapsedTime(&msu, u0, u1);
  const double *M = (const double *)B.pinnedOut.p;
  for (int i = 0; i < P.dim; i++)
    for (int j = i; j < P.dim; j++) I[(size_t)i * rowdim + j] += M[(size_t)i * P.dim + j];
  int err0 = B.pinnedErr[0], err1 = B.pinnedErr[1];
  if (info) {
    info->units = (long long)P.nCentres * P.nPairs;
    info->emitted = -1;
    info->firstFailed = err0 == INT_MAX ? -1 : err0;
    info->values = (long long)P.nCentres * P.centreStride;
    info->msGpu = ms;
    info->msUnitKernel = msu;
    info->h2dBytes = B.h2dBytes;
    info->d2hBytes = (long long)mb + 8;
  }
  if (err1) { set_error("a shell radius did not converge (Newton, 40 steps)"); return 1; }
  return err0 == INT_MAX ? 0 : 2;
}

int run_blocks(const ecpgb_system &s, int mode, double *values, long long *offsets, int *status,
               ecpgb_info *info, Parsed *parsedOut) {
  Engine &E = engine();
  std::unique_lock<std::mutex> lk(E.mu);
  if (!valid_mode(mode)) { set_error("unknown mode %d", mode); return 1; }
  if (E.ensure_init()) return 1;
  Parsed P;
  if (parse_system(s, P)) return 1;
  if (parsedOut) *parsedOut = P;
  const long long nUnits = (long long)P.nCentres * P.nPairs;
  if (nUnits == 0) {
    if (info) { std::memset(info, 0, sizeof *info); info->firstFailed = -1; }
    return 0;
  }
  const DevTables *T = E.get_tables(table_key(P));
  if (!T || E.use_schedules(T, &lk)) return 1;
  JobBuffers &B = E.shared;
  DevJob J;
  if (stage_job(P, T, B, J, mode, E.stream)) return 1;
  const size_t nv = (size_t)P.nCentres * P.centreStride;
  cudaMemsetAsync(B.out.p, 0, sizeof(double) * nv, E.stream);
  cudaEvent_t e0 = E.ev[0], e1 = E.ev[1], u0 = E.ev[2], u1 = E.ev[3];
  cudaEventRecord(e0, E.stream);
  if (run_pipeline(B, J, mode, u0, u1, nullptr, E.stream)) return 1;
  cudaEventRecord(e1, E.stream);
  if (values) cudaMemcpyAsync(values, B.out.p, sizeof(double) * nv, cudaMemcpyDeviceToHost, E.stream);
  std::vector<int> st(nUnits);
  cudaMemcpyAsync(st.data(), B.status.p, sizeof(int) * nUnits, cudaMemcpyDeviceToHost, E.stream);
  cudaMemcpyAsync(B.pinnedErr, B.err.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, E.stream);
  cudaError_t ce = cudaStreamSynchronize(E.stream);
  if (ce != cudaSuccess) { set_error("device error: %s", cudaGetErrorString(ce)); return 1; }
  float ms = 0, msu = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventElapsedTime(&msu, u0, u1);
  long long emitted = 0;
  for (long long u = 0; u < nUnits; u++) {
    if (status) status[u] = st[u];
    if (offsets) offsets[u] = (u / P.nPairs) * P.centreStride + P.pairOff[u % P.nPairs];
    emitted += st[u] != kUnitSkipped;
  }
  int err0 = B.pinnedErr[0], err1 = B.pinnedErr[1];
  if (info) {
    info->units = nUnits;
    info->emitted = emitted;
    info->firstFailed = err0 == INT_MAX ? -1 : err0;
    info->values = (long long)nv;
    info->msGpu = ms;
    info->msUnitKernel = msu;
    info->h2dBytes = B.h2dBytes;
    info->d2hBytes = (long long)(sizeof(double) * nv + sizeof(int) * nUnits);
  }
  if (err1) { set_error("a shell radius did not converge (Newton, 40 steps)"); return 1; }
  return 0;
}

// Energy and nuclear gradient of a density matrix (device-side consumers,
// ecp_grad.cu): the order-0 pipeline for E, the order-1 pipeline for the
// gradient, each contracted with D on the GPU.
int run_gradient(const ecpgb_system &s0, int mode, const double *D, int ldD, double *energy, double *grad) {
  Engine &E = engine();
  std::unique_lock<std::mutex> lk(E.mu);
  if (!valid_mode(mode)) { set_error("unknown mode %d", mode); return 1; }
  if (E.ensure_init()) return 1;
  ecpgb_system s = s0;
  for (int order : {0, 1}) {
    if (order == 0 && !energy) continue;
    if (order == 1 && !grad) continue;
    s.derivative = order;
    Parsed P;
    if (parse_system(s, P)) return 1;
    if (ldD < P.dim) { set_error("ldD %d < basis dimension %d", ldD, P.dim); return 1; }
    const size_t nD = (size_t)P.dim * ldD;
    if (!E.dens.ensure(nD + 1) || !E.gradBuf.ensure(3 * (size_t)P.nAtoms + 1)) {
      set_error("device allocation failed");
      return 1;
    }
    if (P.nCentres == 0 || P.nPairs == 0) {
      if (order == 0) *energy = 0.0;
      else std::memset(grad, 0, sizeof(double) * 3 * P.nAtoms);
      continue;
    }
    const DevTables *T = E.get_tables(table_key(P));
    if (!T || E.use_schedules(T, &lk)) return 1;
    JobBuffers &B = E.shared;
    DevJob J;
    if (stage_job(P, T, B, J, mode, E.stream)) return 1;
    CUDA_OK(cudaMemcpyAsync(E.dens.p, D, sizeof(double) * nD, cudaMemcpyHostToDevice, E.stream));
    if (run_pipeline(B, J, mode, nullptr, nullptr, nullptr, E.stream)) return 1;
    if (order == 0) {
      launch_energy(B.mat.p, P.dim, E.dens.p, ldD, E.gradBuf.p, E.stream);
      CUDA_OK(cudaMemcpyAsync(energy, E.gradBuf.p, sizeof(double), cudaMemcpyDeviceToHost, E.stream));
    } else {
      CUDA_OK(cudaMemsetAsync(E.gradBuf.p, 0, sizeof(double) * 3 * P.nAtoms, E.stream));
      launch_gradient(J, E.dens.p, ldD, E.gradBuf.p, E.stream);
      CUDA_OK(cudaMemcpyAsync(grad, E.gradBuf.p, sizeof(double) * 3 * P.nAtoms, cudaMemcpyDeviceToHost,
                              E.stream));
    }
    cudaError_t ce = cudaStreamSynchronize(E.stream);
    if (ce != cudaSuccess) { set_error("device error: %s", cudaGetErrorString(ce)); return 1; }
  }
  return 0;
}

// Spherical layout of the blocks: per pair entry 2 nsph(lpa) nsph(lpb)
// values (lpa, lpb the l of the blocks the entry hands out).
static long long sph_layout(const Parsed &P, std::vector<long long> &off) {
  off.assign(P.nPairs, 0);
  long long o = 0;
  for (int px = 0; px < P.nPairs; px++) {
    off[px] = o;
    int la = P.shL[P.pairA[px]], lb = P.shL[P.pairB[px]], ha = 0, hb = 0, lpa = la, lpb = lb;
    if (P.deriv) {
      shift_pair(P.deriv, P.pairShift[px], ha, hb);
      if (la + ha < 0 || lb + hb < 0) continue;
      shift_block_l(P.deriv, la, lb, ha, hb, lpa, lpb);
    }
    o += 2LL * (2 * lpa + 1) * (2 * lpb + 1);
  }
  return o;
}

int layout_sph(const ecpgb_system &s, long long *nUnits, long long *nValues) {
  Parsed P;
  if (parse_system(s, P)) return 1;
  std::vector<long long> off;
  const long long stride = sph_layout(P, off);
  if (nUnits) *nUnits = (long long)P.nCentres * P.nPairs;
  if (nValues) *nValues = (long long)P.nCentres * stride;
  return 0;
}

// Every block in real spherical harmonics (src/transformations.c:29-87),
// transformed on the GPU; the ecpgb_blocks contract otherwise.
int run_blocks_sph(const ecpgb_system &s, int mode, double *values, long long *offsets, int *status) {
  Engine &E = engine();
  std::unique_lock<std::mutex> lk(E.mu);
  if (!valid_mode(mode)) { set_error("unknown mode %d", mode); return 1; }
  if (E.ensure_init()) return 1;
  Parsed P;
  if (parse_system(s, P)) return 1;
  const long long nUnits = (long long)P.nCentres * P.nPairs;
  if (nUnits == 0) return 0;
  const DevTables *T = E.get_tables(table_key(P));
  if (!T || E.use_schedules(T, &lk)) return 1;
  JobBuffers &B = E.shared;
  DevJob J;
  if (stage_job(P, T, B, J, mode, E.stream)) return 1;
  std::vector<long long> off;
  const long long stride = sph_layout(P, off);
  const size_t nv = (size_t)P.nCentres * stride;
  if (!B.sphOff.ensure(off.size() + 1) || !B.sout.ensure(nv + 1)) {
    set_error("device allocation failed");
    return 1;
  }
  CUDA_OK(cudaMemcpyAsync(B.sphOff.p, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, E.stream));
  CUDA_OK(cudaMemsetAsync(B.sout.p, 0, sizeof(double) * nv, E.stream));
  if (run_pipeline(B, J, mode, nullptr, nullptr, nullptr, E.stream)) return 1;
  launch_to_sph(J, T->c2s.p, B.sphOff.p, stride, B.sout.p, E.stream);
  if (values) CUDA_OK(cudaMemcpyAsync(values, B.sout.p, sizeof(double) * nv, cudaMemcpyDeviceToHost, E.stream));
  std::vector<int> st(nUnits);
  CUDA_OK(cudaMemcpyAsync(st.data(), B.status.p, sizeof(int) * nUnits, cudaMemcpyDeviceToHost, E.stream));
  cudaError_t ce = cudaStreamSynchronize(E.stream);
  if (ce != cudaSuccess) { set_error("device error: %s", cudaGetErrorString(ce)); return 1; }
  for (long long u = 0; u < nUnits; u++) {
    if (status) status[u] = st[u];
    if (offsets) offsets[u] = (u / P.nPairs) * stride + off[u % P.nPairs];
  }
  return 0;
}

int cart2sph_table(int l, double *out) {
  if (l < 0 || l > kMaxLBasis) { set_error("l %d outside 0..%d", l, kMaxLBasis); return 1; }
  HostTables t;
  build_tables({1, kMaxLBasis, 1024, 1e-12, 1e-14, {}}, t);
  if (t.status) { set_error("table build failed"); return 1; }
  size_t o = 0;
  for (int k = 0; k < l; k++) o += (size_t)(2 * k + 1) * ncart(k);
  std::memcpy(out, t.cart2sph.data() + o, sizeof(double) * (2 * l + 1) * ncart(l));
  return 0;
}

int layout(const ecpgb_system &s, long long *nUnits, long long *nValues) {
  Parsed P;
  if (parse_system(s, P)) return 1;
  if (nUnits) *nUnits = (long long)P.nCentres * P.nPairs;
  if (nValues) *nValues = (long long)P.nCentres * P.centreStride;
  return 0;
}

// ------------------------------------------------------------ resident jobs

struct ResidentJob {
  Parsed P;
  const DevTables *T = nullptr;
  JobBuffers B;
  DevJob J;

  int mode = ECPGB_FP64;
  FastConfig cfg;
  bool useGraph = true;
  // the whole pipeline captured once and replayed per run; gu0/gu1 are
  // recorded inside it around the unit kernel
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t gu0 = nullptr, gu1 = nullptr;
  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
  ~ResidentJob() {
    drop_graph();
    if (gu0) cudaEventDestroy(gu0);
    if (gu1) cudaEventDestroy(gu1);
  }
};

// Captures the job's pipeline into R->graph (engine lock held).
static int capture_graph(Engine &E, ResidentJob *R) {
  if (R->graph) return 0;
  if (!R->gu0) cudaEventCreate(&R->gu0);
  if (!R->gu1) cudaEventCreate(&R->gu1);
  if (R->mode != ECPGB_FP64) fast_prepare();  // function attributes before capture
  cudaGraph_t g = nullptr;
  CUDA_OK(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
  int rc = run_pipeline(R->B, R->J, R->mode, R->gu0, R->gu1, &R->cfg, E.stream);
  cudaError_t ce = cudaStreamEndCapture(E.stream, &g);
  if (rc || ce != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    set_error("pipeline capture failed: %s", cudaGetErrorString(ce));
    return -1;
  }
  ce = cudaGraphInstantiate(&R->graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) {
    R->graph = nullptr;
    set_error("graph instantiation failed: %s", cudaGetErrorString(ce));
    return -1;
  }
  return 0;
}

void *job_create(const ecpgb_system &s, int mode) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  if (!valid_mode(mode)) { set_error("unknown mode %d", mode); return nullptr; }
  if (E.ensure_init()) return nullptr;
  auto *R = new ResidentJob();
  R->mode = mode;
  if (parse_system(s, R->P)) { delete R; return nullptr; }
  if (R->P.nCentres == 0 || R->P.nPairs == 0) { set_error("job has no units"); delete R; return nullptr; }
  R->T = E.get_tables(table_key(R->P));
  if (!R->T || stage_job(R->P, R->T, R->B, R->J, mode, E.stream)) { delete R; return nullptr; }
  R->cfg = E.config_for(R->J.maxLBS, R->J.maxLECP);

  // skipped units are never written: their values read as zero
  cudaMemsetAsync(R->B.out.p, 0, sizeof(double) * (size_t)R->P.nCentres * R->P.centreStride, E.stream);
  if (cudaStreamSynchronize(E.stream) != cudaSuccess) { set_error("staging failed"); delete R; return nullptr; }
  return R;
}

int job_run(void *vj, int nRuns, int flushL2, float *msRun, float *msUnit) {
  Engine &E = engine();
  std::unique_lock<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  if (E.use_schedules(R->T, &lk)) return 1;
  const size_t flushBytes = 256u << 20;
  if (flushL2 && !E.flush.ensure(flushBytes)) { set_error("flush buffer allocation failed"); return 1; }
  if (R->useGraph) {
    // graph replay: the unit-kernel events live inside the graph, so each
    // run is read back before the next replay re-records them
    if (capture_graph(E, R)) return 1;
    cudaEvent_t a0, a1;
    cudaEventCreate(&a0);
    cudaEventCreate(&a1);
    for (int r = 0; r < nRuns; r++) {
      if (flushL2) cudaMemsetAsync(E.flush.p, r & 0xff, flushBytes, E.stream);
      cudaEventRecord(a0, E.stream);
      cudaError_t ce = cudaGraphLaunch(R->graph, E.stream);
      cudaEventRecord(a1, E.stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(E.stream);
      if (ce != cudaSuccess) {
        cudaEventDestroy(a0);
        cudaEventDestroy(a1);
        set_error("device error: %s", cudaGetErrorString(ce));
        return 1;
      }
      float a = 0, b = 0;
      cudaEventElapsedTime(&a, a0, a1);
      cudaEventElapsedTime(&b, R->gu0, R->gu1);
      if (msRun) msRun[r] = a;
      if (msUnit) msUnit[r] = b;
    }
    cudaEventDestroy(a0);
    cudaEventDestroy(a1);
    return 0;
  }
  std::vector<cudaEvent_t> ev(4 * nRuns);
  for (auto &e : ev) cudaEventCreate(&e);
  for (int r = 0; r < nRuns; r++) {
    if (flushL2) cudaMemsetAsync(E.flush.p, r & 0xff, flushBytes, E.stream);
    cudaEventRecord(ev[4 * r], E.stream);
    if (run_pipeline(R->B, R->J, R->mode, ev[4 * r + 2], ev[4 * r + 3], &R->cfg, E.stream)) return 1;
    cudaEventRecord(ev[4 * r + 1], E.stream);
  }
  cudaError_t ce = cudaStreamSynchronize(E.stream);
  if (ce != cudaSuccess) { set_error("device error: %s", cudaGetErrorString(ce)); return 1; }
  for (int r = 0; r < nRuns; r++) {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev[4 * r], ev[4 * r + 1]);
    cudaEventElapsedTime(&b, ev[4 * r + 2], ev[4 * r + 3]);
    if (msRun) msRun[r] = a;
    if (msUnit) msUnit[r] = b;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  return 0;
}

static ecpgb_launch_config to_c(const FastConfig &c, float ms) {
  int per = 0;
  for (int i = 0; i < kMaxClasses; i++) per |= (c.cls[i] & kClassSet) ? 1 : 0;
  return {c.queue, c.sorted, c.gcap, c.balance, c.screen, per, ms};
}

int job_class_config(void *vj, int n, int *gcap, int *balance) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  for (int i = 0; i < n && i < kMaxClasses; i++) {
    const int v = R->cfg.cls[i];
    if (gcap) gcap[i] = (v & kClassSet) ? (v & 0xfff) : 0;
    if (balance) balance[i] = (v & kClassSet) ? ((v >> 12) & 1) : -1;
  }
  return 0;
}

int job_tune(void *vj, ecpgb_launch_config *chosen, ecpgb_launch_config *trials, int maxTrials, int *nTrials) {
  Engine &E = engine();
  std::unique_lock<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  if (nTrials) *nTrials = 0;
  if (R->mode == ECPGB_FP64) { set_error("the autotuner applies to the batched path only"); return 3; }
  if (E.use_schedules(R->T, &lk)) return 1;
  // candidates: queue or CTA-per-unit, cost order or the reference's, and
  // the step-table cap (pairs per warp against CTAs per SM)
  std::vector<FastConfig> cand;
  auto mk = [](int queue, int sorted, int gcap, int balance) {
    FastConfig c;
    c.queue = queue;
    c.sorted = sorted;
    c.gcap = gcap;
    c.balance = balance;
    return c;
  };
  for (int gcap : {45, 64, 33})
    for (int queue : {1, 0}) cand.push_back(mk(queue, 1, gcap, 1));
  cand.push_back(mk(0, 0, 45, 1));
  cand.push_back(mk(1, 1, 45, 0));
  for (int gcap : {45, 64}) cand.push_back(mk(1, 2, gcap, 1));
  cand.push_back(mk(1, 2, 45, 0));
  FastConfig noScreen = mk(1, 1, 45, 1);
  noScreen.screen = 0;
  cand.push_back(noScreen);
  const size_t flushBytes = 256u << 20;
  if (!E.flush.ensure(flushBytes)) { set_error("flush buffer allocation failed"); return 1; }
  cudaEvent_t u0, u1;
  cudaEventCreate(&u0);
  cudaEventCreate(&u1);
  float best = 1e30f;
  FastConfig bestCfg = R->cfg;
  int n = 0;
  for (const FastConfig &c : cand) {
    if (fast_ctas_per_sm(fast_smem_bytes(R->J.maxLBS, R->J.maxLECP, c.gcap, R->J.maxNP), c.queue) < 1) continue;
    float tot = 0;
    for (int r = 0; r < 3; r++) {
      cudaMemsetAsync(E.flush.p, r & 0xff, flushBytes, E.stream);
      if (run_pipeline(R->B, R->J, R->mode, u0, u1, &c, E.stream)) { cudaEventDestroy(u0); cudaEventDestroy(u1); return 1; }
      cudaError_t ce = cudaStreamSynchronize(E.stream);
      if (ce != cudaSuccess) {
        cudaEventDestroy(u0);
        cudaEventDestroy(u1);
        set_error("device error: %s", cudaGetErrorString(ce));
        return 1;
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, u0, u1);
      if (r) tot += ms;
    }
    float ms = tot / 2;
    if (trials && n < maxTrials) trials[n] = to_c(c, ms);
    n++;
    if (ms < best) { best = ms; bestCfg = c; }
  }
  // per-class refinement on the best persistent configuration: each
  // (la, lb) class takes the type-1 cap (at most the launch's) and balance
  // under which its own units took the fewest cycles, measured with every
  // class on one setting at a time; the combination is kept if the whole job
  // runs faster with it
  if (bestCfg.queue == 1 && E.classCycles.ensure(kMaxClasses)) {
    struct Opt { int gcap, balance; };
    std::vector<Opt> opts;
    for (int gcap : {45, 33})
      for (int bal : {0, 1})
        if (gcap <= bestCfg.gcap) opts.push_back({gcap, bal});
    std::vector<std::vector<unsigned long long>> cyc;
    bool ok = true;
    for (const Opt &o : opts) {
      FastConfig c = bestCfg;
      for (int i = 0; i < kMaxClasses; i++) c.cls[i] = kClassSet | o.gcap | o.balance << 12;
      c.classCycles = E.classCycles.p;
      cudaMemsetAsync(E.flush.p, 0x5a, flushBytes, E.stream);
      cudaMemsetAsync(E.classCycles.p, 0, sizeof(unsigned long long) * kMaxClasses, E.stream);
      std::vector<unsigned long long> h(kMaxClasses, 0);
      if (run_pipeline(R->B, R->J, R->mode, nullptr, nullptr, &c, E.stream) ||
          cudaMemcpyAsync(h.data(), E.classCycles.p, sizeof(unsigned long long) * kMaxClasses,
                          cudaMemcpyDeviceToHost, E.stream) != cudaSuccess ||
          cudaStreamSynchronize(E.stream) != cudaSuccess) {
        ok = false;
        break;
      }
      cyc.push_back(h);
    }
    if (ok && !opts.empty()) {
      FastConfig comb = bestCfg;
      for (int i = 0; i < kMaxClasses; i++) {
        size_t bo = 0;
        for (size_t o = 1; o < opts.size(); o++)
          if (cyc[o][i] < cyc[bo][i]) bo = o;
        comb.cls[i] = kClassSet | opts[bo].gcap | opts[bo].balance << 12;
      }
      float tot = 0;
      for (int r = 0; r < 3 && ok; r++) {
        cudaMemsetAsync(E.flush.p, r & 0xff, flushBytes, E.stream);
        if (run_pipeline(R->B, R->J, R->mode, u0, u1, &comb, E.stream) ||
            cudaStreamSynchronize(E.stream) != cudaSuccess) {
          ok = false;
          break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, u0, u1);
        if (r) tot += ms;
      }
      if (ok) {
        const float ms = tot / 2;
        if (trials && n < maxTrials) trials[n] = to_c(comb, ms);
        n++;
        if (ms < best) { best = ms; bestCfg = comb; }
      }
    }
    if (!ok) {
      cudaEventDestroy(u0);
      cudaEventDestroy(u1);
      set_error("per-class tuning failed: %s", cudaGetErrorString(cudaGetLastError()));
      return 1;
    }
  }
  cudaEventDestroy(u0);
  cudaEventDestroy(u1);
  if (nTrials) *nTrials = n < maxTrials ? n : maxTrials;
  R->cfg = bestCfg;
  R->drop_graph();
  E.tuned[{R->J.maxLBS, R->J.maxLECP}] = bestCfg;
  if (chosen) *chosen = to_c(bestCfg, best);
  return 0;
}

int job_config(void *vj, const ecpgb_launch_config *cfg, ecpgb_launch_config *out) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  if (cfg) {
    if (R->mode == ECPGB_FP64) { set_error("launch configurations apply to the batched path only"); return 3; }
    if (cfg->gcap < 1 || cfg->gcap > 4096) { set_error("gcap %d out of range", cfg->gcap); return 1; }
    FastConfig c;
    c.queue = cfg->queue ? 1 : 0;
    c.sorted = cfg->sorted == 2 ? 2 : (cfg->sorted ? 1 : 0);
    c.gcap = cfg->gcap;
    c.balance = cfg->balance ? 1 : 0;
    c.screen = cfg->screen ? 1 : 0;
    if (fast_ctas_per_sm(fast_smem_bytes(R->J.maxLBS, R->J.maxLECP, c.gcap, R->J.maxNP), c.queue) < 1) {
      set_error("configuration does not fit on an SM");
      return 1;
    }
    R->cfg = c;
    R->drop_graph();
  }
  if (out) *out = to_c(R->cfg, 0.0f);
  return 0;
}

int job_blocks(void *vj, double *values, int *status) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  const size_t nv = (size_t)R->P.nCentres * R->P.centreStride, nu = (size_t)R->P.nCentres * R->P.nPairs;
  if (values) cudaMemcpyAsync(values, R->B.out.p, sizeof(double) * nv, cudaMemcpyDeviceToHost, E.stream);
  if (status) cudaMemcpyAsync(status, R->B.status.p, sizeof(int) * nu, cudaMemcpyDeviceToHost, E.stream);
  cudaError_t ce = cudaStreamSynchronize(E.stream);
  if (ce != cudaSuccess) { set_error("copy failed: %s", cudaGetErrorString(ce)); return 1; }
  return 0;
}

int job_use_graph(void *vj, int on) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  R->useGraph = on != 0;
  if (!R->useGraph) R->drop_graph();
  return 0;
}

int job_matrix(void *vj, int rowdim, double *I) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  auto *R = (ResidentJob *)vj;
  size_t mb = sizeof(double) * (size_t)R->P.dim * R->P.dim;
  std::vector<double> M((size_t)R->P.dim * R->P.dim);
  cudaMemcpyAsync(M.data(), R->B.mat.p, mb, cudaMemcpyDeviceToHost, E.stream);
  if (cudaStreamSynchronize(E.stream) != cudaSuccess) { set_error("copy failed"); return 1; }
  for (int i = 0; i < R->P.dim; i++)
    for (int j = i; j < R->P.dim; j++) I[(size_t)i * rowdim + j] += M[(size_t)i * R->P.dim + j];
  return 0;
}

long long job_units(const void *vj, long long *emitted) {
  auto *R = (const ResidentJob *)vj;
  long long n = (long long)R->P.nCentres * R->P.nPairs;
  if (emitted) {
    Engine &E = engine();
    std::lock_guard<std::mutex> lk(E.mu);
    std::vector<int> st(n);
    cudaMemcpy(st.data(), R->B.status.p, sizeof(int) * n, cudaMemcpyDeviceToHost);
    long long c = 0;
    for (int v : st) c += v != kUnitSkipped;
    *emitted = c;
  }
  return n;
}

int job_launches(const void *vj) {
  // reset, four per-job stages, the unit kernel, the AO scatter (order 0), and
  // with the batched queue launch the three screening kernels
  const auto *R = (const ResidentJob *)vj;
  int n = 6 + (R->P.deriv ? 0 : 1);
  if (R->mode != ECPGB_FP64 && R->cfg.queue && R->cfg.screen) n += 3;
  return n;
}

void job_free(void *vj) {
  Engine &E = engine();
  std::lock_guard<std::mutex> lk(E.mu);
  cudaStreamSynchronize(E.stream);
  delete (ResidentJob *)vj;
}

}  // namespace ecpgb

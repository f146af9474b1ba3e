// ecp_capi.cpp -- the C ABI of libecp_gb300.so.
//
// Drop-in symbols with chrr/libECP's prototypes and semantics:
//   getIntegrals                       src/getIntegrals.h:7-13
//   libECP_init / calculateECPIntegrals / libECP_free   src/libecp.h:15-29
//   newECP / checkECP / getECP / evalECP / ECP_free      src/ecp.h:24-39
// plus the ecpgb_* entry points of libecp_gb300.h.  Every integral is
// computed by the CUDA kernels; without a GPU the calls fail with an error
// (there is no CPU path).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ecp.h"
#include "ecp_host.h"
#include "ecp_tables.h"
#include "getIntegrals.h"
#include "libecp.h"
#include "libecp_gb300.h"

using ecpgb::ncart;

struct _libECPHandle {
  ecpgb_system sys;
  std::vector<int> shellsECP, KECP, lECP;  // ECP arrays are copied, as the reference copies its ECPs
  std::vector<double> nECP, dECP, aECP;
  std::vector<int> ordering;               // copied too (the reference keeps the caller's pointer)
};

struct ecpgb_job {
  void *impl;
};

namespace {

// The engine behind the reference's own entry points (getIntegrals,
// calculateECPIntegrals): the plain FP64 kernels unless the environment
// variable LIBECP_GB300_MODE selects the batched FP64 engine ("fast": the
// same results within 1e-10, several times faster) or the mixed-precision
// mode ("mixed"), so that a host program linked unchanged can switch.
int drop_in_mode() {
  const char *m = std::getenv("LIBECP_GB300_MODE");
  if (!m || !*m || !std::strcmp(m, "fp64")) return ECPGB_FP64;
  if (!std::strcmp(m, "fast")) return ECPGB_FAST;
  if (!std::strcmp(m, "mixed")) return ECPGB_MIXED;
  fprintf(stderr, "libecp_gb300: LIBECP_GB300_MODE=%s is not fp64, fast or mixed; using fp64\n", m);
  return ECPGB_FP64;
}

}  // namespace

extern "C" {

int getIntegrals(int nrAtoms, double *geometry, int *shellsECP, int *KECP, int *lECP, double *nECP,
                 double *dECP, double *aECP, int *shellsBS, int *lBS, int *KBS, double *dBS,
                 double *aBS, int largeGridOrder, double tolerance, double accuracy, int rowdim,
                 double *I) {
  ecpgb_system s = {nrAtoms, geometry, shellsECP, KECP, lECP, nECP, dECP, aECP,
                    shellsBS, lBS, KBS, dBS, aBS, largeGridOrder, tolerance, accuracy};
  int rc = ecpgb::run_matrix(s, drop_in_mode(), rowdim, I, nullptr);
  if (rc == 1 || rc < 0) {
    printf("error initializing libECP\n");
    fprintf(stderr, "libecp_gb300: %s\n", ecpgb::last_error());
    return 1;
  }
  return 0;  // like the reference, quadrature failures are not reported here
}

libECPHandle *libECP_init(int nrAtoms, double *geometry, int *shellsECP, int *lECP, int *KECP,
                          double *nECP, double *dECP, double *aECP, int *shellsBS, int *lBS,
                          int *KBS, double *dBS, double *aBS, int n, int lmax, int *shellOrdering,
                          int largeGridOrder, double tolerance, double accuracy) {
  if (n < 0 || n > 2) {  // the reference's shift table covers orders 0..2 (src/libecp.c:243-248)
    ecpgb::set_error("derivative order %d outside 0..2", n);
    return nullptr;
  }
  if (nrAtoms < 1) return nullptr;
  auto *h = new _libECPHandle();
  int nsh = 0, nt = 0;
  h->shellsECP.assign(shellsECP, shellsECP + nrAtoms);
  for (int i = 0; i < nrAtoms; i++) nsh += shellsECP[i] > 0 ? shellsECP[i] : 0;
  h->lECP.assign(lECP, lECP + nsh);
  h->KECP.assign(KECP, KECP + nsh);
  for (int j = 0; j < nsh; j++) nt += KECP[j];
  h->nECP.assign(nECP, nECP + nt);
  h->dECP.assign(dECP, dECP + nt);
  h->aECP.assign(aECP, aECP + nt);
  h->sys = {nrAtoms, geometry, h->shellsECP.data(), h->KECP.data(), h->lECP.data(), h->nECP.data(),
            h->dECP.data(), h->aECP.data(), shellsBS, lBS, KBS, dBS, aBS, largeGridOrder,
            tolerance, accuracy, n, nullptr, 0};
  if (shellOrdering) {  // triples of shells 0..lmax (src/libecp.c:159-165)
    if (lmax < 0 || lmax > 24) {
      ecpgb::set_error("lmax %d out of range for shellOrdering", lmax);
      delete h;
      return nullptr;
    }
    h->ordering.assign(shellOrdering, shellOrdering + 3 * ((lmax + 1) * (lmax + 2) * (lmax + 3) / 6));
    h->sys.shellOrdering = h->ordering.data();
    h->sys.orderingLmax = lmax;
  }
  ecpgb::Parsed P;
  if (ecpgb::parse_system(h->sys, P)) {
    delete h;
    return nullptr;
  }
  ecpgb::HostTables t;
  ecpgb::build_tables(ecpgb::table_key(P), t);
  if (t.status) {  // e.g. the Bessel series does not converge (src/libecp.c:181-185)
    delete h;
    return nullptr;
  }
  return h;
}

int calculateECPIntegrals(libECPHandle *h, ECPCallback cb, void *args) {
  long long nUnits = 0, nValues = 0;
  if (!h || ecpgb::layout(h->sys, &nUnits, &nValues)) return -1;
  std::vector<double> values(nValues > 0 ? nValues : 1);
  std::vector<long long> offsets(nUnits > 0 ? nUnits : 1);
  std::vector<int> status(nUnits > 0 ? nUnits : 1);
  ecpgb_info info;
  ecpgb::Parsed P;
  if (ecpgb::run_blocks(h->sys, drop_in_mode(), values.data(), offsets.data(), status.data(), &info, &P)) {
    fprintf(stderr, "libecp_gb300: %s\n", ecpgb::last_error());
    return -1;
  }
  std::vector<double> blk;
  int result = 0;
  for (long long u = 0; u < nUnits; u++) {
    int st = status[u];
    if (st == ECPGB_UNIT_SKIPPED) continue;
    int c = (int)(u / P.nPairs), p = (int)(u % P.nPairs);
    int sa = P.pairA[p], sb = P.pairB[p], la = P.shL[sa], lb = P.shL[sb];
    int A = P.shAtom[sa], B = P.shAtom[sb], C = P.ctrAtom[c];
    int ha = 0, hb = 0, lpa = la, lpb = lb;  // derivative shift and the blocks' l
    if (P.deriv) {
      ecpgb::shift_pair(P.deriv, P.pairShift[p], ha, hb);
      ecpgb::shift_block_l(P.deriv, la, lb, ha, hb, lpa, lpb);
    }
    size_t nb = (size_t)ncart(lpa) * ncart(lpb);
    const double *b1 = values.data() + offsets[u];
    blk.assign(b1, b1 + nb);
    cb(A, P.shLocal[sa], la, ha, B, P.shLocal[sb], lb, hb, C, blk.data(), args);
    blk.assign(b1 + nb, b1 + 2 * nb);
    cb(A, P.shLocal[sa], la, ha, B, P.shLocal[sb], lb, hb, C, blk.data(), args);
    if (result == 0 && st == ECPGB_UNIT_WARN_TYPE1) result = 1;
    if (result == 0 && st == ECPGB_UNIT_WARN_TYPE2) result = 2;
  }
  return result;
}

void libECP_free(libECPHandle *h) { delete h; }

// ------------------------------------------------------------ ECP helpers

ECP *newECP(const int L, const int N) {
  ECP *U = (ECP *)malloc(sizeof(ECP));
  U->L = L;
  U->N = N;
  U->U_l = (ECPGauss *)calloc(N > 0 ? N : 1, sizeof(ECPGauss));
  for (int i = 0; i < N; i++) U->U_l[i].l = -1;
  return U;
}

int checkECP(const ECP *U) {
  int l = 0;
  for (int i = 0; i < U->N; i++) {
    const ECPGauss *g = &U->U_l[i];
    if (l > g->l || U->L < g->l) return 1;
    if (l < g->l) l = g->l;
  }
  return 0;
}

int getECP(const ECP *U, const int l, ECPGauss **U_l) {
  int n = 0;
  for (int i = 0; i < U->N; i++) n += U->U_l[i].l == l;
  *U_l = (ECPGauss *)malloc(sizeof(ECPGauss) * (n > 0 ? n : 1));
  for (int i = 0, k = 0; i < U->N; i++)
    if (U->U_l[i].l == l) (*U_l)[k++] = U->U_l[i];
  return n;
}

double evalECP(const ECP *U, const int l, const double r) {
  double pot = 0.0, r2 = r * r;
  for (int i = 0; i < U->N; i++) {
    const ECPGauss *g = &U->U_l[i];
    if (g->l == l) pot += pow(r, g->n) * g->d * exp(-g->a * r2);
  }
  return pot;
}

void ECP_free(ECP *E) {
  if (!E) return;
  free(E->U_l);
  free(E);
}

// ------------------------------------------------------------ ecpgb_*

int ecpgb_layout(const ecpgb_system *s, long long *nUnits, long long *nValues) {
  return s ? ecpgb::layout(*s, nUnits, nValues) : 1;
}

int ecpgb_blocks(const ecpgb_system *s, int mode, double *values, long long *offsets, int *status,
                 ecpgb_info *info) {
  if (!s) return 1;
  return ecpgb::run_blocks(*s, mode, values, offsets, status, info, nullptr) ? 1 : 0;
}

int ecpgb_layout_sph(const ecpgb_system *s, long long *nUnits, long long *nValues) {
  return s ? ecpgb::layout_sph(*s, nUnits, nValues) : 1;
}

int ecpgb_blocks_sph(const ecpgb_system *s, int mode, double *values, long long *offsets, int *status) {
  if (!s) { ecpgb::set_error("null system"); return 1; }
  return ecpgb::run_blocks_sph(*s, mode, values, offsets, status);
}

int ecpgb_cart2sph(int l, double *out) { return out ? ecpgb::cart2sph_table(l, out) : 1; }

int ecpgb_gradient(const ecpgb_system *s, int mode, const double *D, int ldD, double *energy, double *grad) {
  if (!s || !D) { ecpgb::set_error("null system or density matrix"); return 1; }
  return ecpgb::run_gradient(*s, mode, D, ldD, energy, grad);
}

int ecpgb_getIntegrals(const ecpgb_system *s, int mode, int rowdim, double *I, ecpgb_info *info) {
  if (!s) return 1;
  int rc = ecpgb::run_matrix(*s, mode, rowdim, I, info);
  return rc < 0 ? 1 : rc;
}

ecpgb_job *ecpgb_job_create(const ecpgb_system *s, int mode) {
  if (!s) return nullptr;
  void *impl = ecpgb::job_create(*s, mode);
  if (!impl) return nullptr;
  return new ecpgb_job{impl};
}

int ecpgb_job_run(ecpgb_job *j, int nRuns, int flushL2, float *msRun, float *msUnit) {
  return j ? ecpgb::job_run(j->impl, nRuns, flushL2, msRun, msUnit) : 1;
}

int ecpgb_job_matrix(ecpgb_job *j, int rowdim, double *I) {
  return j ? ecpgb::job_matrix(j->impl, rowdim, I) : 1;
}

long long ecpgb_job_units(const ecpgb_job *j, long long *emitted) {
  return j ? ecpgb::job_units(j->impl, emitted) : 0;
}

int ecpgb_job_kernel_launches(const ecpgb_job *j) { return j ? ecpgb::job_launches(j->impl) : 0; }

int ecpgb_job_tune(ecpgb_job *j, ecpgb_launch_config *chosen, ecpgb_launch_config *trials, int maxTrials,
                   int *nTrials) {
  return j ? ecpgb::job_tune(j->impl, chosen, trials, maxTrials, nTrials) : 1;
}

int ecpgb_job_config(ecpgb_job *j, const ecpgb_launch_config *cfg, ecpgb_launch_config *out) {
  return j ? ecpgb::job_config(j->impl, cfg, out) : 1;
}

int ecpgb_job_class_config(ecpgb_job *j, int n, int *gcap, int *balance) {
  return j ? ecpgb::job_class_config(j->impl, n, gcap, balance) : 1;
}

int ecpgb_job_use_graph(ecpgb_job *j, int on) { return j ? ecpgb::job_use_graph(j->impl, on) : 1; }

int ecpgb_job_blocks(ecpgb_job *j, double *values, int *status) {
  return j ? ecpgb::job_blocks(j->impl, values, status) : 1;
}

struct ecpgb_server {
  void *impl;
};

ecpgb_server *ecpgb_server_create(int mode, long long hbmBudgetBytes, int slots) {
  void *impl = ecpgb::server_create(mode, hbmBudgetBytes, slots);
  return impl ? new ecpgb_server{impl} : nullptr;
}

long long ecpgb_server_submit(ecpgb_server *sv, const ecpgb_system *s) {
  if (!sv || !s) { ecpgb::set_error("null server or system"); return -1; }
  return ecpgb::server_submit(sv->impl, *s);
}

int ecpgb_server_poll(ecpgb_server *sv, long long id) { return sv ? ecpgb::server_poll(sv->impl, id) : -1; }

int ecpgb_server_wait(ecpgb_server *sv, long long id, int rowdim, double *I, ecpgb_request_info *info) {
  return sv ? ecpgb::server_wait(sv->impl, id, rowdim, I, info) : 1;
}

int ecpgb_server_get_stats(ecpgb_server *sv, ecpgb_server_stats *st) {
  return sv && st ? ecpgb::server_stats(sv->impl, st) : 1;
}

void ecpgb_server_free(ecpgb_server *sv) {
  if (!sv) return;
  ecpgb::server_free(sv->impl);
  delete sv;
}

void ecpgb_job_free(ecpgb_job *j) {
  if (!j) return;
  ecpgb::job_free(j->impl);
  delete j;
}

int ecpgb_measure_peaks(double *out) { return ecpgb::measure_peaks(out); }

int ecpgb_set_device(int device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    ecpgb::set_error("cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

const char *ecpgb_last_error(void) { return ecpgb::last_error(); }

}  // extern "C"

// ecp_host.h -- host-side types of the engine (parsed job, device buffers).
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <algorithm>
#include <vector>

#include "ecp_engine.h"
#include "libecp_gb300.h"

namespace ecpgb {

const char *last_error();
void set_error(const char *fmt, ...);

// Job description parsed from getIntegrals-style arrays.
struct Parsed {
  int nAtoms = 0, nShells = 0, nPrims = 0, nCentres = 0, nPairs = 0, dim = 0;
  int maxLECP = 0, maxLBS = 0, largeGridOrder = 1024;
  // derivative order and its shifts: the pair list below holds every shell
  // pair nShift times (pair-major, shift-minor, the reference's callback
  // order), pairShift the shift index of each entry
  int deriv = 0, nShift = 1;
  std::vector<int> ordering;  // a caller's Cartesian order (empty: libint's)
  double tol = 1e-12, acc = 1e-14;
  std::vector<double> geom, primA, primD, termN, termD, termA;
  std::vector<int> shL, shK, shP, shAtom, shAO, shLocal, atomMaxL, atomShell0;
  std::vector<int> ctrAtom, ctrL, ctrT0, ctrNT, termL, pairA, pairB, pairShift;
  std::vector<long long> pairOff;
  long long centreStride = 0;
};

int parse_system(const ecpgb_system &s, Parsed &P);

// Derivative shifts (src/libecp.c:240-248): number per order and the pair.
int shift_count(int deriv);
void shift_pair(int deriv, int s, int &shifta, int &shiftb);
// Angular momenta of the blocks a shifted unit hands out: the shifted ones,
// except the order-2 shifts (+1, 0) and (0, +1), whose blocks keep the
// unshifted l (src/libecp.c:356-362).
void shift_block_l(int deriv, int la, int lb, int shifta, int shiftb, int &lpa, int &lpb);
struct TableKey;
TableKey table_key(const Parsed &P);

// The stream on which the calling thread's buffer growth is ordered: with a
// stream set, DBuf grows with cudaFreeAsync / cudaMallocAsync on it, which
// do not wait for the rest of the device (cudaFree does); null: cudaMalloc.
cudaStream_t &alloc_stream();

// Grow-only device buffer.
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t cap = 0;
  bool ensure(size_t n) {
    if (n <= cap) return true;
    cudaStream_t s = alloc_stream();
    if (p) {
      if (s) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
    if ((s ? cudaMallocAsync((void **)&p, n * sizeof(T), s) : cudaMalloc((void **)&p, n * sizeof(T))) !=
        cudaSuccess)
      return false;
    cap = n;
    return true;
  }
  // Releases the memory, ordered on stream s (null: cudaFree).
  void release(cudaStream_t s) {
    if (p) {
      if (s) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
  }
  bool upload(const std::vector<T> &v, cudaStream_t s) {
    if (!ensure(v.size() + 1)) return false;
    if (!v.empty() && cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return false;
    return cudaStreamSynchronize(s) == cudaSuccess;
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
};

// Pinned host buffers retired while an allocation stream was set: freeing
// one (cudaFreeHost) waits for the whole device, so they are kept here until
// free_retired_pinned() runs at a quiet point (the request server's shutdown).
std::vector<void *> &retired_pinned();
void retire_pinned(void *p);
void free_retired_pinned();

// Grow-only pinned host buffer; grows by at least half its size.
struct PinnedBuf {
  char *p = nullptr;
  size_t cap = 0;
  bool ensure(size_t n) {
    if (n <= cap) return true;
    if (p) {
      if (alloc_stream()) retire_pinned(p);
      else cudaFreeHost(p);
    }
    p = nullptr;
    const size_t want = std::max(n, cap + cap / 2);
    cap = 0;
    if (cudaMallocHost((void **)&p, want) != cudaSuccess) return false;
    cap = want;
    return true;
  }
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf &) = delete;
  PinnedBuf &operator=(const PinnedBuf &) = delete;
};

// Device allocations of one job.
struct JobBuffers {
  DBuf<char> in;
  DBuf<double> radius, utab, uL, F, cgeo, usp, ang, out, mat;
  DBuf<int> gridEnd, win, status, err;
  DBuf<unsigned long long> head, liveCount;
  DBuf<int> live, screenBlocks;  // screening stage of the batched path
  DBuf<double> sout;       // spherical blocks
  DBuf<long long> sphOff;  // their per-entry offsets
  PinnedBuf pinned, pinnedOut;
  int *pinnedErr = nullptr;
  size_t smem = 0, smemFast = 0;
  long long h2dBytes = 0;
  JobBuffers() { cudaMallocHost((void **)&pinnedErr, 4 * sizeof(int)); }
  // device bytes held by the buffers
  size_t device_bytes() const {
    return in.cap + 8 * (radius.cap + utab.cap + uL.cap + F.cap + cgeo.cap + usp.cap + ang.cap + out.cap + mat.cap) +
           4 * (gridEnd.cap + win.cap + status.cap + err.cap + live.cap + screenBlocks.cap) +
           8 * (head.cap + liveCount.cap);
  }
  // Releases the device buffers (ordered on stream s); they grow again on use.
  void release(cudaStream_t s) {
    in.release(s);
    for (DBuf<double> *b : {&radius, &utab, &uL, &F, &cgeo, &usp, &ang, &out, &mat, &sout}) b->release(s);
    for (DBuf<int> *b : {&gridEnd, &win, &status, &err, &live, &screenBlocks}) b->release(s);
    head.release(s);
    liveCount.release(s);
    sphOff.release(s);
  }
  ~JobBuffers() {
    if (pinnedErr) cudaFreeHost(pinnedErr);
  }
};

int run_matrix(const ecpgb_system &s, int mode, int rowdim, double *I, ecpgb_info *info);
int run_blocks(const ecpgb_system &s, int mode, double *values, long long *offsets, int *status,
               ecpgb_info *info, Parsed *parsedOut);
int layout(const ecpgb_system &s, long long *nUnits, long long *nValues);
int run_gradient(const ecpgb_system &s, int mode, const double *D, int ldD, double *energy, double *grad);
int layout_sph(const ecpgb_system &s, long long *nUnits, long long *nValues);
int run_blocks_sph(const ecpgb_system &s, int mode, double *values, long long *offsets, int *status);
int cart2sph_table(int l, double *out);
void *job_create(const ecpgb_system &s, int mode);
int job_run(void *j, int nRuns, int flushL2, float *msRun, float *msUnit);
int job_matrix(void *j, int rowdim, double *I);
long long job_units(const void *j, long long *emitted);
int job_launches(const void *j);
void job_free(void *j);
int job_tune(void *j, ecpgb_launch_config *chosen, ecpgb_launch_config *trials, int maxTrials, int *nTrials);
int job_config(void *j, const ecpgb_launch_config *cfg, ecpgb_launch_config *out);
int job_class_config(void *j, int n, int *gcap, int *balance);
int job_use_graph(void *j, int on);
int job_blocks(void *j, double *values, int *status);
int measure_peaks(double *out);

// The engine's lock (serialises every use of the shared __constant__ level
// schedules), and the notice a caller holding it gives after writing those
// schedules itself, so the engine re-uploads its own before its next run.
std::mutex &engine_mutex();
void schedules_overwritten();
// Waits (releasing lk, which holds the engine lock) until no request in
// flight pins the level schedules.
void wait_schedules_unpinned(std::unique_lock<std::mutex> &lk);
int run_matrix_noalloc(const ecpgb_system &s, int rowdim, double *I);

bool valid_mode(int mode);

// ---- internals shared with the request server (ecp_serve.cpp)
struct DevTables;
// Packs P's inputs into B's pinned buffer, copies them to the device on
// `stream` and fills J (B's buffers grow as needed).
int stage_job(const Parsed &P, const DevTables *T, JobBuffers &B, DevJob &J, int mode, cudaStream_t stream);
// Resets the run's words and launches the pipeline of the mode on `stream`;
// cfg null = the tuned configuration for the job's (l, L).
int run_pipeline(JobBuffers &B, const DevJob &J, int mode, cudaEvent_t u0, cudaEvent_t u1,
                 const FastConfig *cfg, cudaStream_t stream);
// Device bytes a job of P will hold (inputs and work arrays).
size_t job_device_bytes(const Parsed &P, int mode);
// With the engine lock held: the tables of the request and, unless requests
// in flight pin other level schedules (returns 4: retry after they finish),
// its schedules made current and pinned.  0 ok, 1 error.
int engine_pin_request(const Parsed &P, const DevTables **T);
// With the engine lock held: releases one pin.
void engine_unpin_request();
// Server objects (ecp_serve.cpp).
void *server_create(int mode, long long budget, int slots);
long long server_submit(void *sv, const ecpgb_system &s);
int server_poll(void *sv, long long id);
int server_wait(void *sv, long long id, int rowdim, double *I, ecpgb_request_info *info);
int server_stats(void *sv, ecpgb_server_stats *st);
void server_free(void *sv);

}  // namespace ecpgb

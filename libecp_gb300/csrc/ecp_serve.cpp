// ecp_serve.cpp -- request server with continuous batching.
//
// Jobs (whole getIntegrals systems) are submitted from any thread and parsed
// on submission.  One worker thread owns the GPU side:
//   * admission in arrival order: the head of the queue starts as soon as a
//     slot is free and the slots' device bytes plus the job's stay within
//     the budget;
//   * each slot is a CUDA stream with grow-only device buffers and pinned
//     staging: the job's inputs go up, the pipeline of the server's mode runs
//     and the AO matrix comes back, all on that stream, so jobs admitted while
//     others are running overlap on the device;
//   * completion is read from the slot's last event; the matrix is copied out
//     of the pinned buffer and the slot is free again;
//   * continuous batching at unit granularity: in the batched modes a served
//     job's persistent CTAs each take at most kServeCtaUnits units and exit,
//     so no job holds the SMs for its whole duration, and jobs below
//     kSmallUnits units run on high-priority streams, whose pending CTAs the
//     hardware places before those of the large jobs -- a small request that
//     arrives while a large one runs starts within one CTA's units.
// The basis-independent tables live in the engine and are shared by every
// job; the level schedules are __constant__ data, so jobs in flight pin them
// and a job whose large grid differs waits until the pins are released.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ecp_engine.h"
#include "ecp_host.h"

namespace ecpgb {

namespace {

constexpr int kServeCtaUnits = 8;            // units a served job's CTA takes before it exits
constexpr long long kSmallUnits = 100000;    // (centre, pair) units below which a job is small

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  long long id = 0;
  Parsed P;
  size_t need = 0;  // device bytes estimate
  int state = 0;    // 0 queued, 1 running, 2 done, 3 failed
  int rc = 0;       // like ecpgb_getIntegrals: 0 ok, 2 unit warnings, 1 failure
  std::string err;
  std::vector<double> result;  // dim x dim, upper triangle valid
  double tSubmit = 0, tStart = 0, tDone = 0;
  float gpuMs = 0;
  long long deviceBytes = 0;
  int slot = -1, firstFailed = -1;
};

struct Slot {
  JobBuffers B;
  DevJob J{};
  cudaStream_t stream = nullptr;   // the stream of the current job
  cudaStream_t hi = nullptr, lo = nullptr;  // high- and low-priority streams
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::shared_ptr<Request> req;
};

struct Server {
  int mode = ECPGB_FAST, device = 0;
  size_t budget = 0;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;  // queue, request map, counters
  std::condition_variable cv;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<long long, std::shared_ptr<Request>> reqs;
  long long nextId = 0, submitted = 0, completed = 0, failed = 0;
  std::vector<size_t> slotBytes;  // device bytes per slot, as the worker last saw them
  int inflight = 0, maxInflight = 0;
  bool stop = false;
  std::thread worker;

  size_t held() const {
    size_t b = 0;
    for (auto &s : slots) b += s->B.device_bytes();
    return b;
  }

  void finish(Request &r, int state) {
    std::lock_guard<std::mutex> lk(mu);
    r.state = state;
    r.tDone = now_ms();
    if (state == 2) completed++;
    else failed++;
    cv.notify_all();
  }

  // Starts r on slot k.  0 started, 4 the level schedules are pinned by
  // other jobs (retry later), 1 failed (r is finished as failed).
  int start(int k, const std::shared_ptr<Request> &r) {
    Slot &s = *slots[k];
    const DevTables *T = nullptr;
    std::unique_lock<std::mutex> lk(engine_mutex());
    int rc = engine_pin_request(r->P, &T);
    if (rc == 4) return 4;
    if (rc) {
      r->err = last_error();
      finish(*r, 3);
      return 1;
    }
    r->tStart = now_ms();
    r->slot = k;
    const long long units = (long long)r->P.nCentres * r->P.nPairs;
    s.stream = units < kSmallUnits ? s.hi : s.lo;
    // buffer growth ordered on the slot's stream: admitting a job never
    // waits for the jobs running on the other slots
    alloc_stream() = s.stream;
    bool ok = stage_job(r->P, T, s.B, s.J, mode, s.stream) == 0;
    alloc_stream() = nullptr;
    s.J.ctaUnits = kServeCtaUnits;
    ok = ok && cudaEventRecord(s.e0, s.stream) == cudaSuccess;
    ok = ok && run_pipeline(s.B, s.J, mode, nullptr, nullptr, nullptr, s.stream) == 0;
    const size_t mb = sizeof(double) * (size_t)r->P.dim * r->P.dim;
    alloc_stream() = s.stream;  // a retired pinned buffer is freed later, not here
    ok = ok && s.B.pinnedOut.ensure(mb);
    alloc_stream() = nullptr;
    ok = ok && cudaMemcpyAsync(s.B.pinnedOut.p, s.B.mat.p, mb, cudaMemcpyDeviceToHost, s.stream) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s.B.pinnedErr, s.B.err.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s.stream) ==
                   cudaSuccess;
    ok = ok && cudaEventRecord(s.e1, s.stream) == cudaSuccess;
    if (!ok) {
      r->err = last_error();
      cudaStreamSynchronize(s.stream);
      engine_unpin_request();
      finish(*r, 3);
      return 1;
    }
    r->deviceBytes = (long long)s.B.device_bytes();
    s.req = r;
    {
      std::lock_guard<std::mutex> g(mu);
      slotBytes[k] = (size_t)r->deviceBytes;
      r->state = 1;
    }
    return 0;
  }

  // Retires slot k if its job is done.  Returns 1 when it retired one.
  int retire(int k) {
    Slot &s = *slots[k];
    if (!s.req) return 0;
    cudaError_t ce = cudaEventQuery(s.e1);
    if (ce == cudaErrorNotReady) return 0;
    std::shared_ptr<Request> r = std::move(s.req);
    s.req = nullptr;
    {
      std::lock_guard<std::mutex> lk(engine_mutex());
      engine_unpin_request();
    }
    if (ce != cudaSuccess) {
      r->err = std::string("device error: ") + cudaGetErrorString(ce);
      finish(*r, 3);
      return 1;
    }
    cudaEventElapsedTime(&r->gpuMs, s.e0, s.e1);
    const size_t n = (size_t)r->P.dim * r->P.dim;
    r->result.assign((const double *)s.B.pinnedOut.p, (const double *)s.B.pinnedOut.p + n);
    const int err0 = s.B.pinnedErr[0], err1 = s.B.pinnedErr[1];
    r->firstFailed = err0 == INT_MAX ? -1 : err0;
    if (err1) {
      r->err = "a shell radius did not converge (Newton, 40 steps)";
      finish(*r, 3);
      return 1;
    }
    r->rc = err0 == INT_MAX ? 0 : 2;
    finish(*r, 2);
    return 1;
  }

  void loop() {
    cudaSetDevice(device);
    for (;;) {
      int busy = 0;
      for (size_t k = 0; k < slots.size(); k++) {
        if (retire((int)k)) {
          std::lock_guard<std::mutex> lk(mu);
          inflight--;
        }
        busy += slots[k]->req != nullptr;
      }
      // admission, in arrival order
      for (;;) {
        std::shared_ptr<Request> r;
        {
          std::lock_guard<std::mutex> lk(mu);
          if (queue.empty()) break;
          r = queue.front();
        }
        // the free slot that fits best: the smallest that holds the job
        // without growing, else the largest
        int k = -1;
        for (size_t i = 0; i < slots.size(); i++) {
          if (slots[i]->req) continue;
          if (k < 0) { k = (int)i; continue; }
          const size_t bi = slots[i]->B.device_bytes(), bk = slots[k]->B.device_bytes();
          const bool fi = bi >= r->need, fk = bk >= r->need;
          if ((fi && (!fk || bi < bk)) || (!fi && !fk && bi > bk)) k = (int)i;
        }
        if (k < 0) break;
        size_t mine = slots[k]->B.device_bytes();
        if (r->need > budget) {
          {
            std::lock_guard<std::mutex> lk(mu);
            queue.pop_front();
          }
          r->err = "job needs more device memory than the server's budget";
          finish(*r, 3);
          continue;
        }
        // over the budget: release the buffers of idle slots, largest first
        while (held() - mine + std::max(mine, r->need) > budget) {
          int v = -1;
          for (size_t i = 0; i < slots.size(); i++)
            if ((int)i != k && !slots[i]->req && slots[i]->B.device_bytes() > 0 &&
                (v < 0 || slots[i]->B.device_bytes() > slots[v]->B.device_bytes()))
              v = (int)i;
          if (v < 0) break;
          slots[v]->B.release(slots[v]->stream);
          std::lock_guard<std::mutex> lk(mu);
          slotBytes[v] = 0;
        }
        if (held() - mine + std::max(mine, r->need) > budget) break;  // wait for memory
        int rc = start(k, r);
        if (rc == 4) break;  // other level schedules in flight
        {
          std::lock_guard<std::mutex> lk(mu);
          queue.pop_front();
          if (rc == 0) {
            inflight++;
            maxInflight = std::max(maxInflight, inflight);
            busy++;
          }
        }
      }
      std::unique_lock<std::mutex> lk(mu);
      if (stop && queue.empty() && inflight == 0) break;
      if (inflight == 0 && queue.empty()) cv.wait(lk, [&] { return stop || !queue.empty(); });
      else if (busy) cv.wait_for(lk, std::chrono::microseconds(50));
      else cv.wait_for(lk, std::chrono::microseconds(200));
    }
  }
};

}  // namespace

void *server_create(int mode, long long budget, int nSlots) {
  if (!valid_mode(mode)) {
    set_error("unknown mode %d", mode);
    return nullptr;
  }
  if (nSlots < 1 || nSlots > 64 || budget <= 0) {
    set_error("slots must be 1..64 and the budget positive");
    return nullptr;
  }
  int nDev = 0;
  if (cudaGetDeviceCount(&nDev) != cudaSuccess || nDev < 1) {
    set_error("no CUDA device: the ECP engine runs on the GPU only");
    return nullptr;
  }
  auto *S = new Server();
  S->mode = mode;
  S->budget = (size_t)budget;
  cudaGetDevice(&S->device);
  for (int k = 0; k < nSlots; k++) {
    auto s = std::make_unique<Slot>();
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (cudaStreamCreateWithPriority(&s->hi, cudaStreamNonBlocking, greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s->lo, cudaStreamNonBlocking, least) != cudaSuccess ||
        cudaEventCreate(&s->e0) != cudaSuccess || cudaEventCreate(&s->e1) != cudaSuccess) {
      set_error("stream or event creation failed");
      delete S;
      return nullptr;
    }
    s->stream = s->lo;
    S->slots.push_back(std::move(s));
  }
  S->slotBytes.assign(nSlots, 0);
  S->worker = std::thread([S] { S->loop(); });
  return S;
}

long long server_submit(void *sv, const ecpgb_system &s) {
  auto *S = (Server *)sv;
  auto r = std::make_shared<Request>();
  if (parse_system(s, r->P)) return -1;
  if (r->P.nCentres == 0 || r->P.nPairs == 0) {
    set_error("job has no units");
    return -1;
  }
  r->need = job_device_bytes(r->P, S->mode);
  r->tSubmit = now_ms();
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) {
    set_error("server is shutting down");
    return -1;
  }
  r->id = S->nextId++;
  S->reqs[r->id] = r;
  S->queue.push_back(r);
  S->submitted++;
  S->cv.notify_all();
  return r->id;
}

int server_poll(void *sv, long long id) {
  auto *S = (Server *)sv;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end() || it->second->state == 3) return -1;
  return it->second->state == 2 ? 1 : 0;
}

int server_wait(void *sv, long long id, int rowdim, double *I, ecpgb_request_info *info) {
  auto *S = (Server *)sv;
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) {
      set_error("unknown request %lld", id);
      return 1;
    }
    r = it->second;
    S->cv.wait(lk, [&] { return r->state >= 2; });
    S->reqs.erase(id);
  }
  if (info) {
    info->units = (long long)r->P.nCentres * r->P.nPairs;
    info->values = (long long)r->P.nCentres * r->P.centreStride;
    info->msQueued = r->tStart > 0 ? r->tStart - r->tSubmit : r->tDone - r->tSubmit;
    info->msLatency = r->tDone - r->tSubmit;
    info->msGpu = r->gpuMs;
    info->deviceBytes = r->deviceBytes;
    info->slot = r->slot;
    info->firstFailed = r->firstFailed;
  }
  if (r->state == 3) {
    set_error("%s", r->err.c_str());
    return 1;
  }
  if (rowdim < r->P.dim) {
    set_error("rowdim %d < basis dimension %d", rowdim, r->P.dim);
    return 1;
  }
  const int n = r->P.dim;
  if (I)
    for (int i = 0; i < n; i++)
      for (int j = i; j < n; j++) I[(size_t)i * rowdim + j] += r->result[(size_t)i * n + j];
  return r->rc;
}

int server_stats(void *sv, ecpgb_server_stats *st) {
  auto *S = (Server *)sv;
  std::lock_guard<std::mutex> lk(S->mu);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->failed = S->failed;
  st->queued = (long long)S->queue.size();
  st->inflight = S->inflight;
  st->deviceBytesHeld = 0;
  for (size_t b : S->slotBytes) st->deviceBytesHeld += (long long)b;
  st->budget = (long long)S->budget;
  st->slots = (int)S->slots.size();
  st->maxInflight = S->maxInflight;
  return 0;
}

void server_free(void *sv) {
  auto *S = (Server *)sv;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  for (auto &s : S->slots) {
    for (cudaStream_t st : {s->hi, s->lo})
      if (st) cudaStreamSynchronize(st);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    for (cudaStream_t st : {s->hi, s->lo})
      if (st) cudaStreamDestroy(st);
  }
  delete S;
  free_retired_pinned();
}

}  // namespace ecpgb

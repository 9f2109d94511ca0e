// Serving loop with continuous batching (no counterpart in the reference).
//
// A request is a small ragged batch (host arrays a, b, c, d in FP32, x out
// in FP64, row offsets).  The scheduler thread
//   * admits queued requests in arrival order while their HBM footprint fits
//     the budget and a stream slot is free, coalescing them into one ragged
//     batch (up to max_batch_rows rows);
//   * runs each batch on its own stream: stream-ordered cudaMallocAsync, host
//     -> device copies, an asynchronous plan upload, the refined ragged solve
//     (FP32 solves, FP64 residual and accumulation, `sweeps` corrections),
//     device -> pinned-host copies of x and of the residual;
//   * is told of completion by a host callback on the stream, copies each
//     request's x out of the pinned buffer, frees the batch's memory
//     (cudaFreeAsync) and budget, and admits more work.
// Batches admitted while others are still on the GPU run concurrently on
// their streams, so new requests do not wait for a whole queue to drain.  A
// batch whose maximum relative residual misses the tightest tolerance of its
// requests gets one more correction sweep (up to max_sweeps) before its
// requests complete.  Each system's arithmetic is independent of what else is
// in its batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "runtime.h"
#include "tridi.h"

extern "C" tridi_status tridi_ragged_plan_upload_async(const void* plan, void* dev_buf, size_t bytes,
                                                       tridi_stream_t stream);

namespace tridi {
namespace {

double now_us() {
  return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
long pad4(long v) { return (v + 3) & ~3L; }
size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

struct Request {
  long long id = 0;
  const float *a = nullptr, *b = nullptr, *c = nullptr, *d = nullptr;
  double* x = nullptr;
  std::vector<long> offsets;  // num_systems + 1, rows of this request
  long rows = 0;
  double tol = 1e-10;
  size_t footprint = 0;
  // results
  int status = -1, sweeps = 0;
  double rel = 0.0, t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
  bool done = false;
};

struct Batch {
  std::vector<Request*> reqs;
  std::vector<long> req_row0;  // first row of each request inside the batch
  long rows = 0, systems = 0;
  size_t bytes = 0;
  int slot = -1;
  int sweeps = 0;
  void* plan = nullptr;
  char* dmem = nullptr;  // one allocation: a, b, c, d, x, workspace, plan, offsets, rel
  float *da = nullptr, *db = nullptr, *dc = nullptr, *dd = nullptr;
  double *dx = nullptr, *drel = nullptr;
  long* doff = nullptr;
  void *dws = nullptr, *dplan = nullptr;
  size_t ws_bytes = 0, plan_bytes = 0;
  std::vector<long> offsets;
};

class Server;

struct Slot {
  cudaStream_t stream = nullptr;
  double* host_x = nullptr;  // pinned staging of x (max_batch_rows)
  double* host_rel = nullptr;
  Batch* batch = nullptr;
  Server* server = nullptr;
  std::atomic<bool> finished{false};
};

class Server {
 public:
  Server(size_t budget, long max_batch_rows, int max_inflight, int sweeps, int max_sweeps)
      : budget_(budget), max_rows_(max_batch_rows), sweeps_(sweeps), max_sweeps_(max_sweeps) {
    slots_.resize(max_inflight);
    for (auto& s : slots_) s = new Slot();
  }

  tridi_status init() {
    cudaError_t e;
    if ((e = cudaGetDevice(&device_)) != cudaSuccess) return cuda_status(e);
    if (tridi_init() != TRIDI_SUCCESS) return TRIDI_ERROR_CUDA;
    for (auto* s : slots_) {
      s->server = this;
      if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
          (e = cudaMallocHost(&s->host_x, sizeof(double) * (size_t)pad4(max_rows_))) != cudaSuccess ||
          (e = cudaMallocHost(&s->host_rel, sizeof(double))) != cudaSuccess)
        return cuda_status(e);
    }
    thread_ = std::thread([this] { loop(); });
    return TRIDI_SUCCESS;
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (thread_.joinable()) thread_.join();
    for (auto* s : slots_) {
      if (s->stream) cudaStreamSynchronize(s->stream);
      if (s->batch) finish_batch(s, /*failed=*/true);
      if (s->host_x) cudaFreeHost(s->host_x);
      if (s->host_rel) cudaFreeHost(s->host_rel);
      if (s->stream) cudaStreamDestroy(s->stream);
      delete s;
    }
    for (auto& kv : all_) delete kv.second;
  }

  static size_t footprint(long rows, long systems) {
    const long r = pad4(rows);
    return (size_t)r * (16 + 8) + tridi_ragged_refine_workspace_bytes(rows, systems) + (size_t)systems * 40 +
           (size_t)(systems + 1) * 8 + 4096;
  }

  tridi_status submit(const float* a, const float* b, const float* c, const float* d, double* x,
                      const long* offsets, int num_systems, double tol, long long* id) {
    if (!a || !b || !c || !d || !x || !offsets || num_systems <= 0 || !id) return TRIDI_ERROR_INVALID_VALUE;
    auto* r = new Request();
    r->a = a; r->b = b; r->c = c; r->d = d; r->x = x; r->tol = tol;
    r->offsets.assign(offsets, offsets + num_systems + 1);
    r->rows = offsets[num_systems] - offsets[0];
    if (offsets[0] != 0 || r->rows <= 0) {
      delete r;
      return TRIDI_ERROR_INVALID_VALUE;
    }
    for (int s = 0; s < num_systems; ++s)
      if (offsets[s + 1] <= offsets[s] || offsets[s + 1] - offsets[s] > 17408) {
        delete r;
        return TRIDI_ERROR_UNSUPPORTED_SIZE;
      }
    r->footprint = footprint(r->rows, num_systems);
    if (r->footprint > budget_ || r->rows > max_rows_) {
      delete r;
      return TRIDI_ERROR_OUT_OF_MEMORY;  // can never be admitted
    }
    r->t_submit = now_us();
    {
      std::lock_guard<std::mutex> l(mu_);
      r->id = ++next_id_;
      all_[r->id] = r;
      queue_.push_back(r);
    }
    cv_.notify_all();
    *id = r->id;
    return TRIDI_SUCCESS;
  }

  tridi_status wait(long long id, int timeout_ms, int* status, int* sweeps, double* rel, double* latency_us) {
    std::unique_lock<std::mutex> l(mu_);
    auto it = all_.find(id);
    if (it == all_.end()) return TRIDI_ERROR_INVALID_VALUE;
    Request* r = it->second;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
    while (!r->done) {
      if (timeout_ms >= 0 && done_cv_.wait_until(l, deadline) == std::cv_status::timeout && !r->done)
        return TRIDI_ERROR_BUSY;
      if (timeout_ms < 0) done_cv_.wait(l);
    }
    if (status) *status = r->status;
    if (sweeps) *sweeps = r->sweeps;
    if (rel) *rel = r->rel;
    if (latency_us) *latency_us = r->t_done - r->t_submit;
    all_.erase(it);
    delete r;
    return TRIDI_SUCCESS;
  }

  void stats(long long* completed, long long* batches, long long* rows, double* max_inflight_seen) {
    std::lock_guard<std::mutex> l(mu_);
    if (completed) *completed = completed_;
    if (batches) *batches = batches_;
    if (rows) *rows = rows_done_;
    if (max_inflight_seen) *max_inflight_seen = max_inflight_seen_;
  }

  // called from the stream's host callback thread: no CUDA calls here
  void notify_finished(Slot* s) {
    s->finished.store(true);
    {
      std::lock_guard<std::mutex> l(mu_);
      ++pending_completions_;
    }
    cv_.notify_all();
  }

 private:
  void loop() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> l(mu_);
    while (true) {
      cv_.wait(l, [this] { return stop_ || pending_completions_ > 0 || (!queue_.empty() && free_slot() >= 0); });
      if (stop_) return;
      pending_completions_ = 0;
      l.unlock();
      for (auto* s : slots_)
        if (s->batch && s->finished.exchange(false)) complete(s);
      l.lock();
      admit(l);
    }
  }

  int free_slot() const {
    for (size_t i = 0; i < slots_.size(); ++i)
      if (!slots_[i]->batch) return (int)i;
    return -1;
  }

  // mu_ held on entry and exit
  void admit(std::unique_lock<std::mutex>& l) {
    while (!queue_.empty()) {
      const int si = free_slot();
      if (si < 0) return;
      auto* b = new Batch();
      while (!queue_.empty()) {
        Request* r = queue_.front();
        const long sys = (long)r->offsets.size() - 1;
        const size_t fp = footprint(b->rows + r->rows, b->systems + sys);
        if (b->rows + r->rows > max_rows_ || used_ + fp > budget_) break;
        b->req_row0.push_back(b->rows);
        b->reqs.push_back(r);
        b->rows += r->rows;
        b->systems += sys;
        queue_.pop_front();
      }
      if (b->reqs.empty()) {  // the head request waits for memory to free up
        delete b;
        return;
      }
      b->bytes = footprint(b->rows, b->systems);
      used_ += b->bytes;
      b->slot = si;
      slots_[si]->batch = b;
      ++batches_;
      int inflight = 0;
      for (auto* s : slots_) inflight += s->batch != nullptr;
      max_inflight_seen_ = std::max(max_inflight_seen_, (double)inflight);
      const double t = now_us();
      for (auto* r : b->reqs) r->t_admit = t;
      l.unlock();
      const tridi_status st = launch(slots_[si], b, sweeps_);
      l.lock();
      if (st != TRIDI_SUCCESS) {
        for (auto* r : b->reqs) {
          r->status = st;
          r->t_done = now_us();
          r->done = true;
        }
        used_ -= b->bytes;
        slots_[si]->batch = nullptr;
        release(b);
        done_cv_.notify_all();
      }
    }
  }

  static void CUDART_CB on_done(void* user) {
    Slot* s = static_cast<Slot*>(user);
    s->server->notify_finished(s);
  }

  tridi_status launch(Slot* s, Batch* b, int sweeps) {
    cudaStream_t st = s->stream;
    cudaError_t e;
    if (!b->dmem) {
      // concatenated offsets and the plan
      b->offsets.assign(1, 0);
      for (auto* r : b->reqs)
        for (size_t k = 1; k < r->offsets.size(); ++k) b->offsets.push_back(b->offsets.back() + r->offsets[k] - r->offsets[k - 1]);
      tridi_status ts = tridi_ragged_plan_create(b->offsets.data(), (int)b->systems, &b->plan);
      if (ts != TRIDI_SUCCESS) return ts;
      const long R = pad4(b->rows);
      b->ws_bytes = tridi_ragged_refine_workspace_bytes(b->rows, b->systems);
      b->plan_bytes = tridi_ragged_plan_device_bytes(b->plan);
      const size_t sizes[] = {align256(4 * R), align256(4 * R), align256(4 * R), align256(4 * R), align256(8 * R),
                              align256(b->ws_bytes), align256(b->plan_bytes),
                              align256(sizeof(long) * (b->systems + 1)), 256};
      size_t total = 0;
      for (size_t v : sizes) total += v;
      if ((e = cudaMallocAsync(reinterpret_cast<void**>(&b->dmem), total, st)) != cudaSuccess) return cuda_status(e);
      char* p = b->dmem;
      b->da = reinterpret_cast<float*>(p); p += sizes[0];
      b->db = reinterpret_cast<float*>(p); p += sizes[1];
      b->dc = reinterpret_cast<float*>(p); p += sizes[2];
      b->dd = reinterpret_cast<float*>(p); p += sizes[3];
      b->dx = reinterpret_cast<double*>(p); p += sizes[4];
      b->dws = p; p += sizes[5];
      b->dplan = p; p += sizes[6];
      b->doff = reinterpret_cast<long*>(p); p += sizes[7];
      b->drel = reinterpret_cast<double*>(p);
      // pad rows of the coefficient arrays are read by the bulk copies: define them
      const size_t tail = (size_t)(R - b->rows) * 4;
      for (float* arr : {b->da, b->db, b->dc, b->dd})
        if (tail && (e = cudaMemsetAsync(arr + b->rows, 0, tail, st)) != cudaSuccess) return cuda_status(e);
      for (size_t q = 0; q < b->reqs.size(); ++q) {
        Request* r = b->reqs[q];
        const size_t off = (size_t)b->req_row0[q], bytes = (size_t)r->rows * 4;
        if ((e = cudaMemcpyAsync(b->da + off, r->a, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(b->db + off, r->b, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(b->dc + off, r->c, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(b->dd + off, r->d, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
          return cuda_status(e);
      }
      if ((e = cudaMemcpyAsync(b->doff, b->offsets.data(), sizeof(long) * (b->systems + 1), cudaMemcpyHostToDevice,
                               st)) != cudaSuccess)
        return cuda_status(e);
      ts = tridi_ragged_plan_upload_async(b->plan, b->dplan, b->plan_bytes, st);
      if (ts != TRIDI_SUCCESS) return ts;
    }
    b->sweeps = sweeps;
    tridi_status ts = tridi_ragged_refine_f32(b->da, b->db, b->dc, b->dd, b->dx, b->plan, b->dplan, b->doff, sweeps,
                                              b->dws, b->ws_bytes, b->drel, st);
    if (ts != TRIDI_SUCCESS) return ts;
    if ((e = cudaMemcpyAsync(s->host_x, b->dx, sizeof(double) * b->rows, cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(s->host_rel, b->drel, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaLaunchHostFunc(st, on_done, s)) != cudaSuccess)
      return cuda_status(e);
    return TRIDI_SUCCESS;
  }

  // scheduler thread, mu_ not held
  void complete(Slot* s) {
    Batch* b = s->batch;
    const double rel = *s->host_rel;
    double tol = 1e300;
    for (auto* r : b->reqs) tol = std::min(tol, r->tol);
    if (!(rel <= tol) && b->sweeps < max_sweeps_ && rel == rel) {
      if (launch(s, b, b->sweeps + 1) == TRIDI_SUCCESS) return;  // one more correction sweep
    }
    for (size_t q = 0; q < b->reqs.size(); ++q) {
      Request* r = b->reqs[q];
      std::memcpy(r->x, s->host_x + b->req_row0[q], sizeof(double) * r->rows);
      r->rel = rel;
      r->sweeps = b->sweeps;
      r->status = rel <= r->tol ? TRIDI_SUCCESS : TRIDI_ERROR_NOT_CONVERGED;
    }
    finish_batch(s, false);
  }

  void finish_batch(Slot* s, bool failed) {
    Batch* b = s->batch;
    const double t = now_us();
    {
      std::lock_guard<std::mutex> l(mu_);
      for (auto* r : b->reqs) {
        if (failed) r->status = TRIDI_ERROR_CUDA;
        r->t_done = t;
        r->done = true;
        ++completed_;
        rows_done_ += r->rows;
      }
      used_ -= b->bytes;
      s->batch = nullptr;
    }
    if (b->dmem) cudaFreeAsync(b->dmem, s->stream);
    release(b);
    done_cv_.notify_all();
  }

  void release(Batch* b) {
    if (b->plan) tridi_ragged_plan_destroy(b->plan);
    delete b;
  }

  size_t budget_, used_ = 0;
  long max_rows_;
  int sweeps_, max_sweeps_;
  int device_ = 0;
  std::vector<Slot*> slots_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Request*> queue_;
  std::unordered_map<long long, Request*> all_;
  long long next_id_ = 0, completed_ = 0, batches_ = 0, rows_done_ = 0;
  double max_inflight_seen_ = 0;
  int pending_completions_ = 0;
  bool stop_ = false;
  std::thread thread_;
};

}  // namespace
}  // namespace tridi

extern "C" {

tridi_status tridi_server_create(size_t hbm_budget_bytes, long max_batch_rows, int max_inflight, int sweeps,
                                 int max_sweeps, void** server) {
  if (!server || hbm_budget_bytes == 0 || max_batch_rows <= 0 || max_inflight <= 0 || sweeps < 0 ||
      max_sweeps < sweeps)
    return TRIDI_ERROR_INVALID_VALUE;
  auto* s = new tridi::Server(hbm_budget_bytes, max_batch_rows, max_inflight, sweeps, max_sweeps);
  tridi_status st = s->init();
  if (st != TRIDI_SUCCESS) {
    delete s;
    return st;
  }
  *server = s;
  return TRIDI_SUCCESS;
}

size_t tridi_server_request_footprint(long rows, long num_systems) {
  return tridi::Server::footprint(rows, num_systems);
}

tridi_status tridi_server_submit(void* server, const float* a, const float* b, const float* c, const float* d,
                                 double* x, const long* offsets, int num_systems, double tol, long long* id) {
  if (!server) return TRIDI_ERROR_INVALID_VALUE;
  return static_cast<tridi::Server*>(server)->submit(a, b, c, d, x, offsets, num_systems, tol, id);
}

tridi_status tridi_server_wait(void* server, long long id, int timeout_ms, int* status, int* sweeps,
                               double* rel_residual, double* latency_us) {
  if (!server) return TRIDI_ERROR_INVALID_VALUE;
  return static_cast<tridi::Server*>(server)->wait(id, timeout_ms, status, sweeps, rel_residual, latency_us);
}

tridi_status tridi_server_stats(void* server, long long* completed, long long* batches, long long* rows,
                                double* max_inflight_seen) {
  if (!server) return TRIDI_ERROR_INVALID_VALUE;
  static_cast<tridi::Server*>(server)->stats(completed, batches, rows, max_inflight_seen);
  return TRIDI_SUCCESS;
}

tridi_status tridi_server_destroy(void* server) {
  delete static_cast<tridi::Server*>(server);
  return TRIDI_SUCCESS;
}

}  // extern "C"

// Serving loop with continuous batching (no counterpart in the reference).
//
// A request is a small ragged batch (host arrays a, b, c, d in FP32, x out
// in FP64, row offsets).  Two kinds of host threads:
//   * the scheduler admits queued requests in arrival order while their HBM
//     footprint fits the budget and a stream slot is idle, coalescing them
//     into one ragged batch (up to max_batch_rows rows), and hands the batch
//     to that slot;
//   * each slot's worker runs its batch on the slot's own stream:
//     stream-ordered allocation from the server's pool, host -> device transfer straight from the
//     callers' arrays, an asynchronous plan upload, the fused refinement
//     (FP32 solves, extended-precision residual and accumulation, `sweeps`
//     corrections), the batch's maximum residual read back, one more sweep
//     while it misses the tightest tolerance of the batch (up to max_sweeps),
//     then device -> host copies straight into each request's x, the memory
//     freed (cudaFreeAsync) and the budget returned.
// Slots work concurrently, so a request that arrives while others are on the
// GPU is admitted as soon as a slot and memory free up and its work overlaps
// theirs on the device.  Each system's arithmetic is independent of what else
// is in its batch.  Host transfers (TRIDI_TUNE_SERVER_COPY): by default,
// cudaMemcpyAsync straight from and to the callers' pageable arrays (on a
// Grace host 80-180 GB/s for copies of 8 MB and more, measured); or staged:
// requests of 2^18 rows or more as above, the smaller ones, packed after
// them, in chunks of 2^20 rows through two pinned buffers per slot, which a
// pool of host threads fills from (and empties into) the callers' arrays
// while the copy engines move the other buffer (it never beat the plain
// copies in measurement, and its host threads make it the more sensitive to
// a busy host); or, where the device can access pageable host memory,
// kernels that read the callers' arrays and write their x directly.
#include <cuda_runtime.h>

#include <algorithm>
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

constexpr long kMaxServedSystemRows = 24480;  // the ragged solver's largest system

double now_us() {
  return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
long pad4(long v) { return (v + 3) & ~3L; }
size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// Per-request copy job of a batch: the caller's host arrays and the
// request's first row inside the batch.
struct CopyJob {
  const float* src[4];
  double* dst;
  long row0;
  long rows;
};

// Host -> device: the GPU reads the callers' (pageable) arrays itself over the
// coherent chip-to-chip link (pageable memory access), one grid row per job.
__global__ void gather_kernel(const CopyJob* jobs, float* da, float* db, float* dc, float* dd) {
  const CopyJob j = jobs[blockIdx.y];
  float* dst[4] = {da + j.row0, db + j.row0, dc + j.row0, dd + j.row0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < j.rows; i += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < 4; ++q) dst[q][i] = j.src[q][i];
  }
}

// Device -> host: x of each request written straight into the caller's array.
__global__ void scatter_kernel(const CopyJob* jobs, const double* dx) {
  const CopyJob j = jobs[blockIdx.y];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < j.rows; i += (long)gridDim.x * blockDim.x)
    j.dst[i] = dx[j.row0 + i];
}

// Host threads that copy between the callers' (pageable) arrays and the
// pinned staging buffers, in pieces, in parallel; the calling thread works
// through the pieces too.
class CopyPool {
 public:
  struct Seg {
    void* dst;
    const void* src;
    size_t bytes;
  };
  explicit CopyPool(int n) {
    for (int i = 0; i < n; ++i) th_.emplace_back([this] { loop(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(const std::vector<Seg>& segs) {
    constexpr size_t kPiece = 1 << 20;
    Job job;
    {
      std::lock_guard<std::mutex> l(mu_);
      for (const Seg& g : segs)
        for (size_t o = 0; o < g.bytes; o += kPiece) {
          q_.push_back(Piece{static_cast<char*>(g.dst) + o, static_cast<const char*>(g.src) + o,
                             std::min(kPiece, g.bytes - o), &job});
          ++job.left;
        }
    }
    cv_.notify_all();
    while (true) {  // help, then wait for the pieces others took
      Piece pc{};
      {
        std::unique_lock<std::mutex> l(mu_);
        if (q_.empty() || q_.front().job != &job) {
          job.cv.wait(l, [&] { return job.left == 0; });
          return;
        }
        pc = q_.front();
        q_.pop_front();
      }
      std::memcpy(pc.dst, pc.src, pc.bytes);
      finish(pc);
    }
  }

 private:
  struct Job {
    long left = 0;
    std::condition_variable cv;
  };
  struct Piece {
    char* dst;
    const char* src;
    size_t bytes;
    Job* job;
  };
  void finish(const Piece& pc) {
    std::lock_guard<std::mutex> l(mu_);
    if (--pc.job->left == 0) pc.job->cv.notify_all();
  }
  void loop() {
    while (true) {
      Piece pc{};
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [this] { return stop_ || !q_.empty(); });
        if (stop_ && q_.empty()) return;
        pc = q_.front();
        q_.pop_front();
      }
      std::memcpy(pc.dst, pc.src, pc.bytes);
      finish(pc);
    }
  }
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<Piece> q_;
  bool stop_ = false;
};

constexpr long kStageRows = 1L << 20;  // rows per pinned staging chunk (16 MB in, 8 MB out)
// Requests of at least this many rows move by cudaMemcpyAsync straight from
// and to the callers' arrays (the driver's pageable path runs at 100-170 GB/s
// from 1 MB per copy up); smaller ones go through the pinned staging.
constexpr long kDirectRows = 1L << 18;

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
};

class Server;

struct Slot {
  Server* server = nullptr;
  cudaStream_t stream = nullptr;
  double* host_rel = nullptr;  // pinned
  float* in_stage[2] = {};     // pinned: a, b, c, d of kStageRows rows each
  double* out_stage[2] = {};   // pinned: x of kStageRows rows
  cudaEvent_t in_done[2] = {}, out_done[2] = {};
  Batch* batch = nullptr;      // set by the scheduler, cleared when done (under the server mutex)
  std::thread worker;
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
    // The server's own stream-ordered pool, keeping up to the budget mapped
    // between batches: the default pool returns its memory at every
    // synchronisation, and re-mapping it per batch cost more than the
    // transfers on some hosts.
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device_;
    if ((e = cudaMemPoolCreate(&mempool_, &props)) != cudaSuccess) return cuda_status(e);
    unsigned long long keep = budget_;
    if ((e = cudaMemPoolSetAttribute(mempool_, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
      return cuda_status(e);
    for (auto* s : slots_) {
      s->server = this;
      if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
          (e = cudaMallocHost(&s->host_rel, sizeof(double))) != cudaSuccess)
        return cuda_status(e);
    }
    int pageable = 0;
    if ((e = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device_)) != cudaSuccess)
      return cuda_status(e);
    // Direct access is opt-in: callers' freshly allocated pages fault on the
    // GPU's first touch, which made it slower than the copy engines in
    // measurement; it pays only for arrays the host has already touched.
    const int mode = tunable(TRIDI_TUNE_SERVER_COPY);
    if (mode == TRIDI_SERVER_COPY_DIRECT && !pageable) return TRIDI_ERROR_UNSUPPORTED_SIZE;
    direct_ = mode == TRIDI_SERVER_COPY_DIRECT;
    staged_ = mode == TRIDI_SERVER_COPY_STAGED;
    if (staged_) {
      for (auto* s : slots_)
        for (int k = 0; k < 2; ++k)
          if ((e = cudaMallocHost(&s->in_stage[k], sizeof(float) * 4 * kStageRows)) != cudaSuccess ||
              (e = cudaMallocHost(&s->out_stage[k], sizeof(double) * kStageRows)) != cudaSuccess ||
              (e = cudaEventCreateWithFlags(&s->in_done[k], cudaEventDisableTiming)) != cudaSuccess ||
              (e = cudaEventCreateWithFlags(&s->out_done[k], cudaEventDisableTiming)) != cudaSuccess)
            return cuda_status(e);
      const unsigned hw = std::thread::hardware_concurrency();
      pool_ = new CopyPool(std::max(2, std::min(8, (int)(hw ? hw / 2 : 4))));
    }
    for (auto* s : slots_) s->worker = std::thread([this, s] { work(s); });
    scheduler_ = std::thread([this] { schedule(); });
    return TRIDI_SUCCESS;
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (scheduler_.joinable()) scheduler_.join();
    for (auto* s : slots_)
      if (s->worker.joinable()) s->worker.join();
    delete pool_;
    for (auto* s : slots_) {
      for (int k = 0; k < 2; ++k) {
        if (s->in_stage[k]) cudaFreeHost(s->in_stage[k]);
        if (s->out_stage[k]) cudaFreeHost(s->out_stage[k]);
        if (s->in_done[k]) cudaEventDestroy(s->in_done[k]);
        if (s->out_done[k]) cudaEventDestroy(s->out_done[k]);
      }
      if (s->host_rel) cudaFreeHost(s->host_rel);
      if (s->stream) cudaStreamDestroy(s->stream);
      delete s;
    }
    if (mempool_) cudaMemPoolDestroy(mempool_);
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
      if (offsets[s + 1] <= offsets[s] || offsets[s + 1] - offsets[s] > kMaxServedSystemRows) {
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
      if (timeout_ms >= 0) {
        if (done_cv_.wait_until(l, deadline) == std::cv_status::timeout && !r->done) return TRIDI_ERROR_BUSY;
      } else {
        done_cv_.wait(l);
      }
    }
    if (status) *status = r->status;
    if (sweeps) *sweeps = r->sweeps;
    if (rel) *rel = r->rel;
    if (latency_us) *latency_us = r->t_done - r->t_submit;
    all_.erase(it);
    delete r;
    return TRIDI_SUCCESS;
  }

  // Host microseconds spent by the slot workers, summed over batches, per
  // phase: plan build, allocation + host->device copies issued, solve (up to
  // the residual read-back), device->host copies, free.
  void phase_us(double* out, int n) {
    std::lock_guard<std::mutex> l(mu_);
    for (int i = 0; i < n && i < kPhases; ++i) out[i] = phase_us_[i];
  }

  void stats(long long* completed, long long* batches, long long* rows, double* max_inflight_seen) {
    std::lock_guard<std::mutex> l(mu_);
    if (completed) *completed = completed_;
    if (batches) *batches = batches_;
    if (rows) *rows = rows_done_;
    if (max_inflight_seen) *max_inflight_seen = max_inflight_seen_;
  }

 private:
  // ---- scheduler thread ----
  void schedule() {
    std::unique_lock<std::mutex> l(mu_);
    while (true) {
      cv_.wait(l, [this] { return stop_ || (!queue_.empty() && idle_slot() >= 0); });
      if (stop_) return;
      if (!admit()) {
        // the head request waits for memory: sleep until a batch completes
        const long long seen = batches_done_;
        cv_.wait(l, [this, seen] { return stop_ || batches_done_ != seen; });
      }
    }
  }

  int idle_slot() const {
    for (size_t i = 0; i < slots_.size(); ++i)
      if (!slots_[i]->batch) return (int)i;
    return -1;
  }

  // mu_ held.  Forms one batch for an idle slot; false when the head request
  // does not fit the memory left.
  bool admit() {
    const int si = idle_slot();
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
    if (b->reqs.empty()) {
      delete b;
      return false;
    }
    if (staged_) {  // large requests first, the staged ones in one contiguous row range after them
      std::stable_partition(b->reqs.begin(), b->reqs.end(), [](const Request* r) { return r->rows >= kDirectRows; });
      long row = 0;
      for (size_t q = 0; q < b->reqs.size(); ++q) {
        b->req_row0[q] = row;
        row += b->reqs[q]->rows;
      }
    }
    b->bytes = footprint(b->rows, b->systems);
    used_ += b->bytes;
    ++batches_;
    const double t = now_us();
    for (auto* r : b->reqs) r->t_admit = t;
    slots_[si]->batch = b;
    int inflight = 0;
    for (auto* s : slots_) inflight += s->batch != nullptr;
    max_inflight_seen_ = std::max(max_inflight_seen_, (double)inflight);
    cv_.notify_all();  // wakes the slot's worker
    return true;
  }

  // ---- slot workers ----
  void work(Slot* s) {
    cudaSetDevice(device_);
    while (true) {
      Batch* b = nullptr;
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [this, s] { return stop_ || s->batch != nullptr; });
        if (!s->batch) return;  // stopping, nothing assigned
        b = s->batch;
      }
      int sweeps = 0;
      double rel = 0.0;
      const tridi_status st = run(s, b, &sweeps, &rel);
      finish(s, b, st, sweeps, rel);
    }
  }

  // Runs one batch to completion on the slot's stream (this thread blocks on
  // its own stream only).
  tridi_status run(Slot* s, Batch* b, int* sweeps_out, double* rel_out) {
    cudaStream_t st = s->stream;
    cudaError_t e;
    double ph[kPhases] = {};
    double t = now_us();
    auto lap = [&](int k) {
      const double u = now_us();
      ph[k] += u - t;
      t = u;
    };
    std::vector<long> offsets(1, 0);
    for (auto* r : b->reqs)
      for (size_t k = 1; k < r->offsets.size(); ++k)
        offsets.push_back(offsets.back() + r->offsets[k] - r->offsets[k - 1]);
    void* plan = nullptr;
    tridi_status ts = tridi_ragged_plan_create_refine(offsets.data(), (int)b->systems, &plan);
    if (ts != TRIDI_SUCCESS) return ts;
    lap(0);
    const long R = pad4(b->rows);
    const size_t ws_bytes = tridi_ragged_refine_workspace_bytes(b->rows, b->systems);
    const size_t plan_bytes = tridi_ragged_plan_device_bytes(plan);
    std::vector<CopyJob> jobs(b->reqs.size());
    long max_rows = 0;
    for (size_t q = 0; q < b->reqs.size(); ++q) {
      Request* r = b->reqs[q];
      jobs[q] = CopyJob{{r->a, r->b, r->c, r->d}, r->x, b->req_row0[q], r->rows};
      max_rows = std::max(max_rows, r->rows);
    }
    const size_t sizes[] = {align256(4 * R), align256(4 * R), align256(4 * R), align256(4 * R),
                            align256(8 * R), align256(ws_bytes), align256(plan_bytes), 256,
                            align256(sizeof(CopyJob) * jobs.size())};
    size_t total = 0;
    for (size_t v : sizes) total += v;
    char* dmem = nullptr;
    if ((e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&dmem), total, mempool_, st)) != cudaSuccess) {
      tridi_ragged_plan_destroy(plan);
      return cuda_status(e);
    }
    char* p = dmem;
    float* da = reinterpret_cast<float*>(p); p += sizes[0];
    float* db = reinterpret_cast<float*>(p); p += sizes[1];
    float* dc = reinterpret_cast<float*>(p); p += sizes[2];
    float* dd = reinterpret_cast<float*>(p); p += sizes[3];
    double* dx = reinterpret_cast<double*>(p); p += sizes[4];
    void* dws = p; p += sizes[5];
    void* dplan = p; p += sizes[6];
    double* drel = reinterpret_cast<double*>(p); p += sizes[7];
    CopyJob* djobs = reinterpret_cast<CopyJob*>(p);
    const dim3 cgrid((unsigned)std::min<long>((max_rows + 255) / 256, 64), (unsigned)jobs.size());
    auto body = [&]() -> tridi_status {
      // pad rows of the coefficient arrays are read by the bulk copies: define them
      const size_t tail = (size_t)(R - b->rows) * 4;
      for (float* arr : {da, db, dc, dd})
        if (tail && (e = cudaMemsetAsync(arr + b->rows, 0, tail, st)) != cudaSuccess) return cuda_status(e);
      if (direct_) {
        if ((e = cudaMemcpyAsync(djobs, jobs.data(), sizeof(CopyJob) * jobs.size(), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
          return cuda_status(e);
        gather_kernel<<<cgrid, 256, 0, st>>>(djobs, da, db, dc, dd);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
      } else if (staged_) {
        // large requests straight from the callers' arrays; the rest in chunks
        // of kStageRows rows through two pinned buffers: the pool fills one
        // while the copy engine drains the other
        long s0 = 0;  // first staged row
        for (size_t q = 0; q < b->reqs.size() && b->reqs[q]->rows >= kDirectRows; ++q) {
          Request* r = b->reqs[q];
          const size_t off = (size_t)b->req_row0[q], bytes = (size_t)r->rows * 4;
          if ((e = cudaMemcpyAsync(da + off, r->a, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
              (e = cudaMemcpyAsync(db + off, r->b, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
              (e = cudaMemcpyAsync(dc + off, r->c, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
              (e = cudaMemcpyAsync(dd + off, r->d, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return cuda_status(e);
          s0 = b->req_row0[q] + r->rows;
        }
        std::vector<CopyPool::Seg> segs;
        for (long r0 = s0, k = 0; r0 < b->rows; r0 += kStageRows, ++k) {
          const long r1 = std::min(b->rows, r0 + kStageRows);
          float* buf = s->in_stage[k & 1];
          if (k >= 2 && (e = cudaEventSynchronize(s->in_done[k & 1])) != cudaSuccess) return cuda_status(e);
          segs.clear();
          for (size_t q = 0; q < b->reqs.size(); ++q) {
            Request* r = b->reqs[q];
            const long lo = std::max(r0, b->req_row0[q]), hi = std::min(r1, b->req_row0[q] + r->rows);
            if (lo >= hi) continue;
            const float* src[4] = {r->a, r->b, r->c, r->d};
            for (int a = 0; a < 4; ++a)
              segs.push_back({buf + a * kStageRows + (lo - r0), src[a] + (lo - b->req_row0[q]),
                              sizeof(float) * (hi - lo)});
          }
          pool_->run(segs);
          float* dst[4] = {da, db, dc, dd};
          for (int a = 0; a < 4; ++a)
            if ((e = cudaMemcpyAsync(dst[a] + r0, buf + a * kStageRows, sizeof(float) * (r1 - r0),
                                     cudaMemcpyHostToDevice, st)) != cudaSuccess)
              return cuda_status(e);
          if ((e = cudaEventRecord(s->in_done[k & 1], st)) != cudaSuccess) return cuda_status(e);
        }
      } else {
        for (size_t q = 0; q < b->reqs.size(); ++q) {
          Request* r = b->reqs[q];
          const size_t off = (size_t)b->req_row0[q], bytes = (size_t)r->rows * 4;
          if ((e = cudaMemcpyAsync(da + off, r->a, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
              (e = cudaMemcpyAsync(db + off, r->b, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
              (e = cudaMemcpyAsync(dc + off, r->c, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
              (e = cudaMemcpyAsync(dd + off, r->d, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return cuda_status(e);
        }
      }
      tridi_status t = tridi_ragged_plan_upload_async(plan, dplan, plan_bytes, st);
      if (t != TRIDI_SUCCESS) return t;
      lap(1);
      double tol = 1e300;
      for (auto* r : b->reqs) tol = std::min(tol, r->tol);
      for (int sweeps = sweeps_;; ++sweeps) {
        t = tridi_ragged_refine_f32(da, db, dc, dd, dx, plan, dplan, nullptr, sweeps, dws, ws_bytes, drel, st);
        if (t != TRIDI_SUCCESS) return t;
        if ((e = cudaMemcpyAsync(s->host_rel, drel, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
          return cuda_status(e);
        *rel_out = *s->host_rel;
        *sweeps_out = sweeps;
        if (*rel_out <= tol || !(*rel_out == *rel_out) || sweeps >= max_sweeps_) break;
      }
      lap(2);
      if (direct_) {
        scatter_kernel<<<cgrid, 256, 0, st>>>(djobs, dx);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
      } else if (staged_) {
        // large requests straight into the callers' arrays; for the staged
        // range, chunk k's copy engine transfer overlaps the pool's copy-out
        // of chunk k-1
        long s0 = 0;
        for (size_t q = 0; q < b->reqs.size() && b->reqs[q]->rows >= kDirectRows; ++q) {
          Request* r = b->reqs[q];
          if ((e = cudaMemcpyAsync(r->x, dx + b->req_row0[q], sizeof(double) * r->rows, cudaMemcpyDeviceToHost,
                                   st)) != cudaSuccess)
            return cuda_status(e);
          s0 = b->req_row0[q] + r->rows;
        }
        std::vector<CopyPool::Seg> segs;
        const long nchunks = (b->rows - s0 + kStageRows - 1) / kStageRows;
        auto copy_out = [&](long k) {
          const long r0 = s0 + k * kStageRows, r1 = std::min(b->rows, r0 + kStageRows);
          const double* buf = s->out_stage[k & 1];
          segs.clear();
          for (size_t q = 0; q < b->reqs.size(); ++q) {
            Request* r = b->reqs[q];
            const long lo = std::max(r0, b->req_row0[q]), hi = std::min(r1, b->req_row0[q] + r->rows);
            if (lo < hi) segs.push_back({r->x + (lo - b->req_row0[q]), buf + (lo - r0), sizeof(double) * (hi - lo)});
          }
          pool_->run(segs);
        };
        for (long k = 0; k < nchunks; ++k) {
          const long r0 = s0 + k * kStageRows, r1 = std::min(b->rows, r0 + kStageRows);
          if ((e = cudaMemcpyAsync(s->out_stage[k & 1], dx + r0, sizeof(double) * (r1 - r0), cudaMemcpyDeviceToHost,
                                   st)) != cudaSuccess ||
              (e = cudaEventRecord(s->out_done[k & 1], st)) != cudaSuccess)
            return cuda_status(e);
          if (k >= 1) {
            if ((e = cudaEventSynchronize(s->out_done[(k - 1) & 1])) != cudaSuccess) return cuda_status(e);
            copy_out(k - 1);
          }
        }
        if (nchunks > 0) {
          if ((e = cudaEventSynchronize(s->out_done[(nchunks - 1) & 1])) != cudaSuccess) return cuda_status(e);
          copy_out(nchunks - 1);
        }
      } else {
        for (size_t q = 0; q < b->reqs.size(); ++q) {
          Request* r = b->reqs[q];
          if ((e = cudaMemcpyAsync(r->x, dx + b->req_row0[q], sizeof(double) * r->rows, cudaMemcpyDeviceToHost,
                                   st)) != cudaSuccess)
            return cuda_status(e);
        }
      }
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_status(e);
      lap(3);
      return TRIDI_SUCCESS;
    };
    ts = body();
    cudaFreeAsync(dmem, st);
    cudaStreamSynchronize(st);  // the plan's host arrays feed the upload: keep them until it ran
    tridi_ragged_plan_destroy(plan);
    lap(4);
    {
      std::lock_guard<std::mutex> l(mu_);
      for (int k = 0; k < kPhases; ++k) phase_us_[k] += ph[k];
    }
    return ts;
  }

  void finish(Slot* s, Batch* b, tridi_status st, int sweeps, double rel) {
    const double t = now_us();
    {
      std::lock_guard<std::mutex> l(mu_);
      for (auto* r : b->reqs) {
        r->rel = rel;
        r->sweeps = sweeps;
        r->status = st != TRIDI_SUCCESS ? st : (rel <= r->tol ? TRIDI_SUCCESS : TRIDI_ERROR_NOT_CONVERGED);
        r->t_done = t;
        r->done = true;
        ++completed_;
        rows_done_ += r->rows;
      }
      used_ -= b->bytes;
      s->batch = nullptr;
      ++batches_done_;
    }
    delete b;
    cv_.notify_all();
    done_cv_.notify_all();
  }

  size_t budget_, used_ = 0;
  long max_rows_;
  int sweeps_, max_sweeps_;
  int device_ = 0;
  cudaMemPool_t mempool_ = nullptr;
  std::vector<Slot*> slots_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Request*> queue_;
  std::unordered_map<long long, Request*> all_;
  long long next_id_ = 0, completed_ = 0, batches_ = 0, batches_done_ = 0, rows_done_ = 0;
  double max_inflight_seen_ = 0;
  bool direct_ = false;  // the GPU reads and writes the callers' host arrays itself
  bool staged_ = false;  // pinned double-buffered staging filled by the copy pool
  CopyPool* pool_ = nullptr;
  static constexpr int kPhases = 5;
  double phase_us_[kPhases] = {};
  bool stop_ = false;
  std::thread scheduler_;
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

tridi_status tridi_server_phase_times(void* server, double* us, int n) {
  if (!server || !us || n < 0) return TRIDI_ERROR_INVALID_VALUE;
  static_cast<tridi::Server*>(server)->phase_us(us, n);
  return TRIDI_SUCCESS;
}

tridi_status tridi_server_destroy(void* server) {
  delete static_cast<tridi::Server*>(server);
  return TRIDI_SUCCESS;
}

}  // extern "C"

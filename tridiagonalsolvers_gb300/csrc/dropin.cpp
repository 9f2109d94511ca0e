// The reference's host launchers (include/tridi_dropin.h) on the GB300
// kernels.  Host pointers in, host pointers out, synchronous.
//
// Per call: the batch is cut into chunks of whole systems; every chunk's
// host->device copies go back to back on a copy-in stream, its solve on a
// compute stream after an event of its copies, its device->host copy on a
// copy-out stream after an event of its solve.  So the host->device engine
// (the bound: about 4/5 of the bytes) never waits behind a device->host copy,
// and the copies of one chunk overlap the solve of another.
// Device buffers come from a persistent per-device workspace (grown on
// demand, never shrunk until tridi_dropin_release), not from a cudaMalloc
// and cudaFree per call as in cr_app.cu:20-24,61-65.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>

#include "runtime.h"
#include "tridi.h"
#include "tridi_dropin.h"

namespace tridi {

// Device work of one chunk (implemented by the kernel translation units).
template <class T>
tridi_status dropin_device_solve(int algo, const T* a, const T* b, const T* c, const T* d, T* x, int n, int m,
                                 int param, void* ws, size_t ws_bytes, cudaStream_t s);

namespace {

constexpr int kMaxChunks = 64;
constexpr int kTimedLaunches = 50;  // the reference's numIterations (common.h:14)
struct Workspace {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream[3] = {nullptr, nullptr, nullptr};  // copy-in, compute, copy-out
  cudaEvent_t in_done[kMaxChunks] = {};
  cudaEvent_t solved[kMaxChunks] = {};
};
constexpr int kMaxDev = 64;
Workspace g_ws[kMaxDev];
std::mutex g_mu;

cudaError_t ensure_workspace(Workspace& w, size_t bytes) {
  cudaError_t e;
  if (!w.stream[0]) {
    for (auto& s : w.stream)
      if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return e;
    for (int k = 0; k < kMaxChunks; ++k) {
      if ((e = cudaEventCreateWithFlags(&w.in_done[k], cudaEventDisableTiming)) != cudaSuccess) return e;
      if ((e = cudaEventCreateWithFlags(&w.solved[k], cudaEventDisableTiming)) != cudaSuccess) return e;
    }
  }
  if (w.bytes >= bytes) return cudaSuccess;
  if (w.ptr) {
    for (auto& s : w.stream) cudaStreamSynchronize(s);
    cudaFree(w.ptr);
    w.ptr = nullptr;
    w.bytes = 0;
  }
  if ((e = cudaMalloc(&w.ptr, bytes)) != cudaSuccess) return e;
  w.bytes = bytes;
  return cudaSuccess;
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// What a host pointer is: `view` = the device's address of host memory that
// is pinned and mapped into its address space (cudaHostAlloc,
// cudaHostRegister with mapping), else null; `pageable` = ordinary host
// memory, neither pinned nor device memory.  One query a pointer.
template <class P>
P* host_view(P* p, bool& pageable) {
  cudaPointerAttributes at{};
  pageable = false;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // unregistered memory on older drivers: not an error of the call
    return nullptr;
  }
  pageable = at.type == cudaMemoryTypeUnregistered;
  return at.type == cudaMemoryTypeHost ? static_cast<P*>(at.devicePointer) : nullptr;
}

// True when device `dev` reads and writes pageable host memory coherently
// through the host's own page tables (address translation services, as on
// Grace hosts): then the solver can work on malloc'd arrays at their own
// addresses.  Queried once per device (callers hold g_mu).
bool pageable_direct(int dev) {
  static signed char known[kMaxDev] = {};  // 0 not yet asked, 1 yes, -1 no
  if (known[dev] == 0) {
    int access = 0, host_tables = 0;
    const bool ok = cudaDeviceGetAttribute(&access, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
                    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
                        cudaSuccess;
    if (!ok) cudaGetLastError();
    known[dev] = ok && access == 1 && host_tables == 1 ? 1 : -1;
  }
  return known[dev] == 1;
}

// Extra device scratch the algorithm needs for m systems of size n.
template <class T>
size_t algo_scratch(int algo, int n, int m, int param);

// Stages the batch through the chunk pipeline.  The chunks' solves are
// ordered on the one compute stream, so they share one scratch slice, sized
// for a full chunk -- or for the whole batch when `whole_batch_scratch` is
// set (the timing path relaunches the device work on all m systems at once).
template <class T>
tridi_status host_solve(int algo, const T* a, const T* b, const T* c, const T* d, T* x, int n, int m, int param,
                        bool whole_batch_scratch = false) {
  if (!a || !b || !c || !d || !x || n <= 0 || m <= 0) return TRIDI_ERROR_INVALID_VALUE;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev < 0 || dev >= kMaxDev) return TRIDI_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> lock(g_mu);
  Workspace& w = g_ws[dev];

  // Arrays that are pinned and mapped: the solver reads a..d and writes x in
  // place over the host link.  The same bytes cross it as with staging
  // copies, but no chunk pipeline fills and drains, and no copy waits for
  // the copy engine behind another.  The same for ordinary pageable arrays
  // where the device reaches them through the host's page tables.  The
  // kernels then read with plain loads (g_host_mapped_io); pcrGauss, whose
  // larger sizes take the partition and large-system solvers, always stages.
  const int in_place = tunable(TRIDI_TUNE_DROPIN_MAPPED);
  if (!whole_batch_scratch && algo != TRIDI_DROPIN_PCR_THOMAS && in_place != 2) {
    bool pa, pb, pc, pd, px;
    const T *va = host_view(a, pa), *vb = host_view(b, pb), *vc = host_view(c, pc), *vd = host_view(d, pd);
    T* vx = host_view(x, px);
    if (!(va && vb && vc && vd && vx) && in_place != 3 && pa && pb && pc && pd && px && pageable_direct(dev)) {
      va = a; vb = b; vc = c; vd = d; vx = x;
    }
    if (va && vb && vc && vd && vx) {
      e = ensure_workspace(w, 0);
      if (e != cudaSuccess) return cuda_status(e);
      g_host_mapped_io = true;
      tridi_status st = dropin_device_solve<T>(algo, va, vb, vc, vd, vx, n, m, param, nullptr, 0, w.stream[1]);
      g_host_mapped_io = false;
      const cudaError_t es = cudaStreamSynchronize(w.stream[1]);
      if (st == TRIDI_SUCCESS && es != cudaSuccess) st = cuda_status(es);
      return st;
    }
  }

  // Chunks of whole systems, at most 64: 8 MiB per coefficient array from
  // pinned memory, 64 MiB from pageable memory (whose copies the driver
  // stages synchronously, so they overlap little and gain from size: 1.96
  // against 2.40 ms for the 65536 x 256 batch), or TRIDI_TUNE_DROPIN_CHUNK KiB.
  const size_t sys_bytes = (size_t)n * sizeof(T);
  const int chunk_kib = tunable(TRIDI_TUNE_DROPIN_CHUNK);
  size_t chunk_bytes = chunk_kib > 0 ? (size_t)chunk_kib << 10 : (size_t)8 << 20;
  if (chunk_kib <= 0) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, a) != cudaSuccess) cudaGetLastError();
    else if (at.type == cudaMemoryTypeUnregistered) chunk_bytes = (size_t)64 << 20;
  }
  long per = (long)(chunk_bytes / sys_bytes);
  if (per < 1) per = 1;
  if (per * kMaxChunks < m) per = (m + kMaxChunks - 1) / kMaxChunks;
  if (per > m) per = m;
  const size_t arr = align256((size_t)m * sys_bytes);
  size_t ws_bytes = align256(algo_scratch<T>(algo, n, (int)per, param));
  if (whole_batch_scratch) {
    const size_t whole = align256(algo_scratch<T>(algo, n, m, param));
    if (whole > ws_bytes) ws_bytes = whole;
  }
  if ((e = ensure_workspace(w, 5 * arr + ws_bytes)) != cudaSuccess) return cuda_status(e);
  char* base = static_cast<char*>(w.ptr);
  T* da = reinterpret_cast<T*>(base);
  T* db = reinterpret_cast<T*>(base + arr);
  T* dc = reinterpret_cast<T*>(base + 2 * arr);
  T* dd = reinterpret_cast<T*>(base + 3 * arr);
  T* dx = reinterpret_cast<T*>(base + 4 * arr);
  void* ws = base + 5 * arr;

  tridi_status st = TRIDI_SUCCESS;
  cudaStream_t s_in = w.stream[0], s_comp = w.stream[1], s_out = w.stream[2];
  for (long s0 = 0, k = 0; s0 < m; s0 += per, ++k) {
    const long cnt = (m - s0) < per ? (m - s0) : per;
    const size_t off = (size_t)s0 * n, bytes = (size_t)cnt * sys_bytes;
    if ((e = cudaMemcpyAsync(da + off, a + off, bytes, cudaMemcpyHostToDevice, s_in)) != cudaSuccess ||
        (e = cudaMemcpyAsync(db + off, b + off, bytes, cudaMemcpyHostToDevice, s_in)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dc + off, c + off, bytes, cudaMemcpyHostToDevice, s_in)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dd + off, d + off, bytes, cudaMemcpyHostToDevice, s_in)) != cudaSuccess ||
        (e = cudaEventRecord(w.in_done[k], s_in)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(s_comp, w.in_done[k], 0)) != cudaSuccess) {
      st = cuda_status(e);
      break;
    }
    st = dropin_device_solve<T>(algo, da + off, db + off, dc + off, dd + off, dx + off, n, (int)cnt, param, ws,
                                ws_bytes, s_comp);
    if (st != TRIDI_SUCCESS) break;
    if ((e = cudaEventRecord(w.solved[k], s_comp)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(s_out, w.solved[k], 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync(x + off, dx + off, bytes, cudaMemcpyDeviceToHost, s_out)) != cudaSuccess) {
      st = cuda_status(e);
      break;
    }
  }
  cudaError_t es[3];
  for (int q = 0; q < 3; ++q) es[q] = cudaStreamSynchronize(w.stream[q]);
  for (int q = 0; q < 3 && st == TRIDI_SUCCESS; ++q)
    if (es[q] != cudaSuccess) st = cuda_status(es[q]);
  return st;
}

const char* algo_name(int algo) {
  static const char* names[] = {"cr", "pcr", "crpcr", "crNBC", "crpcrNBC", "crNBC", "pcrGauss"};
  return algo >= 0 && algo < 7 ? names[algo] : "?";
}

// numIterations (common.h:14) = 50 timed launches of the device work on the
// staged batch, printed like cr_app.cu:48 / pcrGauss_app.cu.  Runs after a
// full host_solve that staged the inputs into the workspace, on the compute
// stream, with CUDA events; every launch's status is checked.
template <class T>
tridi_status time_device_work(int algo, int n, int m, int param, float* ms_per_launch) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  std::lock_guard<std::mutex> lock(g_mu);
  Workspace& w = g_ws[dev];
  const size_t arr = align256((size_t)m * n * sizeof(T));
  const size_t need = align256(algo_scratch<T>(algo, n, m, param));
  if (!w.ptr || w.bytes < 5 * arr + need) return TRIDI_ERROR_WORKSPACE_TOO_SMALL;
  char* base = static_cast<char*>(w.ptr);
  cudaStream_t s = w.stream[1];
  cudaEvent_t ev[2] = {nullptr, nullptr};
  tridi_status st = TRIDI_SUCCESS;
  if ((e = cudaEventCreate(&ev[0])) != cudaSuccess || (e = cudaEventCreate(&ev[1])) != cudaSuccess ||
      (e = cudaEventRecord(ev[0], s)) != cudaSuccess)
    st = cuda_status(e);
  for (int i = 0; i < kTimedLaunches && st == TRIDI_SUCCESS; ++i)
    st = dropin_device_solve<T>(algo, reinterpret_cast<T*>(base), reinterpret_cast<T*>(base + arr),
                                reinterpret_cast<T*>(base + 2 * arr), reinterpret_cast<T*>(base + 3 * arr),
                                reinterpret_cast<T*>(base + 4 * arr), n, m, param, base + 5 * arr,
                                w.bytes - 5 * arr, s);
  if (st == TRIDI_SUCCESS && (e = cudaEventRecord(ev[1], s)) != cudaSuccess) st = cuda_status(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess && st == TRIDI_SUCCESS) st = cuda_status(e);
  if (st == TRIDI_SUCCESS) {
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, ev[0], ev[1])) != cudaSuccess) st = cuda_status(e);
    *ms_per_launch = ms / kTimedLaunches;
  }
  for (auto& v : ev)
    if (v) cudaEventDestroy(v);
  return st;
}

// The C++ drop-ins: reference error behaviour (print, then exit like
// CUDA_SAFE_CALL, unless TRIDI_DROPIN_NO_EXIT=1) and, with
// TRIDI_DROPIN_TIMING=1, the reference's timing line.
template <class T>
void dropin(int algo, T* a, T* b, T* c, T* d, T* x, int n, int m, int param) {
  const char* timing = std::getenv("TRIDI_DROPIN_TIMING");
  tridi_status st = TRIDI_SUCCESS;
  if (timing && timing[0] == '1') {
    float ms = 0.f;
    st = host_solve<T>(algo, a, b, c, d, x, n, m, param, /*whole_batch_scratch=*/true);
    if (st == TRIDI_SUCCESS) st = time_device_work<T>(algo, n, m, param, &ms);
    if (st == TRIDI_SUCCESS) {
      if (algo == TRIDI_DROPIN_PCR_THOMAS)
        printf("pcrGauss: GPU kernel time: %f ms\n", ms);
      else
        printf("%s: numSystems: %d, systemSize: %d, GPU kernel time: %f ms\n", algo_name(algo), m, n, ms);
      fflush(stdout);
    }
  }
  // the solve whose x the caller gets (as the reference re-runs its kernel on
  // fresh inputs after timing, cr_app.cu:50-56)
  if (st == TRIDI_SUCCESS) st = host_solve<T>(algo, a, b, c, d, x, n, m, param);
  if (st != TRIDI_SUCCESS) {
    fprintf(stderr, "tridi: %s(systemSize=%d, numSystems=%d) failed: %s (cuda error %d)\n", algo_name(algo), n, m,
            tridi_status_string(st), tridi_last_cuda_error());
    const char* noexit = std::getenv("TRIDI_DROPIN_NO_EXIT");
    if (!(noexit && noexit[0] == '1')) std::exit(1);
  }
}

}  // namespace

template <class T>
size_t algo_scratch_bytes(int algo, int n, int m, int param);

namespace {
template <class T>
size_t algo_scratch(int algo, int n, int m, int param) {
  return algo_scratch_bytes<T>(algo, n, m, param);
}
}  // namespace

}  // namespace tridi

using tridi::dropin;

void cr(float* a, float* b, float* c, float* d, float* x, int n, int m) { dropin<float>(TRIDI_DROPIN_CR, a, b, c, d, x, n, m, 0); }
void cr(double* a, double* b, double* c, double* d, double* x, int n, int m) { dropin<double>(TRIDI_DROPIN_CR, a, b, c, d, x, n, m, 0); }
void pcr(float* a, float* b, float* c, float* d, float* x, int n, int m) { dropin<float>(TRIDI_DROPIN_PCR, a, b, c, d, x, n, m, 0); }
void pcr(double* a, double* b, double* c, double* d, double* x, int n, int m) { dropin<double>(TRIDI_DROPIN_PCR, a, b, c, d, x, n, m, 0); }
void crpcr(float* a, float* b, float* c, float* d, float* x, int n, int m, int rest) { dropin<float>(TRIDI_DROPIN_CRPCR, a, b, c, d, x, n, m, rest); }
void crpcr(double* a, double* b, double* c, double* d, double* x, int n, int m, int rest) { dropin<double>(TRIDI_DROPIN_CRPCR, a, b, c, d, x, n, m, rest); }
void crNBC(float* a, float* b, float* c, float* d, float* x, int n, int m) { dropin<float>(TRIDI_DROPIN_CR_NBC, a, b, c, d, x, n, m, 0); }
void crNBC(double* a, double* b, double* c, double* d, double* x, int n, int m) { dropin<double>(TRIDI_DROPIN_CR_NBC, a, b, c, d, x, n, m, 0); }
void crpcrNBC(float* a, float* b, float* c, float* d, float* x, int n, int m, int rest) { dropin<float>(TRIDI_DROPIN_CRPCR_NBC, a, b, c, d, x, n, m, rest); }
void crpcrNBC(double* a, double* b, double* c, double* d, double* x, int n, int m, int rest) { dropin<double>(TRIDI_DROPIN_CRPCR_NBC, a, b, c, d, x, n, m, rest); }
void crNBC32(float* a, float* b, float* c, float* d, float* x, int n, int m) { dropin<float>(TRIDI_DROPIN_CR_NBC32, a, b, c, d, x, n, m, 0); }
void crNBC32(double* a, double* b, double* c, double* d, double* x, int n, int m) { dropin<double>(TRIDI_DROPIN_CR_NBC32, a, b, c, d, x, n, m, 0); }
void pcrGaussWrapper(float* a, float* b, float* c, float* d, float* x, int n, int m, int g) { dropin<float>(TRIDI_DROPIN_PCR_THOMAS, a, b, c, d, x, n, m, g); }
void pcrGaussWrapper(double* a, double* b, double* c, double* d, double* x, int n, int m, int g) { dropin<double>(TRIDI_DROPIN_PCR_THOMAS, a, b, c, d, x, n, m, g); }

extern "C" {

tridi_status tridi_dropin_solve_f32(int algo, const float* a, const float* b, const float* c, const float* d,
                                    float* x, int n, int m, int param) {
  return tridi::host_solve<float>(algo, a, b, c, d, x, n, m, param);
}
tridi_status tridi_dropin_solve_f64(int algo, const double* a, const double* b, const double* c, const double* d,
                                    double* x, int n, int m, int param) {
  return tridi::host_solve<double>(algo, a, b, c, d, x, n, m, param);
}
int tridi_dropin_pageable_in_place(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= tridi::kMaxDev) {
    cudaGetLastError();
    return 0;
  }
  std::lock_guard<std::mutex> lock(tridi::g_mu);
  return tridi::pageable_direct(dev) ? 1 : 0;
}
}  // extern "C"

namespace tridi {
namespace {
template <class T>
tridi_status write_result(const T* x, int m, int n, const char* path) {
  if (!x || !path || m < 0 || n < 0) return TRIDI_ERROR_INVALID_VALUE;
  std::ofstream f(path);
  if (!f) return TRIDI_ERROR_INVALID_VALUE;
  const long total = (long)m * n;
  for (long i = 0; i < total; ++i) {
    if (i % n == 0) f << "***The following is the result of the equation set " << i / n << "\n";
    f << x[i] << "\n";
  }
  return f ? TRIDI_SUCCESS : TRIDI_ERROR_INVALID_VALUE;
}
}  // namespace
}  // namespace tridi

extern "C" {

tridi_status tridi_write_result_file_f32(const float* x, int m, int n, const char* path) {
  return tridi::write_result(x, m, n, path);
}
tridi_status tridi_write_result_file_f64(const double* x, int m, int n, const char* path) {
  return tridi::write_result(x, m, n, path);
}

tridi_status tridi_dropin_release(void) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return tridi::cuda_status(e);
  std::lock_guard<std::mutex> lock(tridi::g_mu);
  tridi::Workspace& w = tridi::g_ws[dev];
  for (auto& s : w.stream)
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
      s = nullptr;
    }
  for (int k = 0; k < tridi::kMaxChunks; ++k) {
    if (w.in_done[k]) cudaEventDestroy(w.in_done[k]);
    if (w.solved[k]) cudaEventDestroy(w.solved[k]);
    w.in_done[k] = w.solved[k] = nullptr;
  }
  if (w.ptr) cudaFree(w.ptr);
  w.ptr = nullptr;
  w.bytes = 0;
  return TRIDI_SUCCESS;
}

}  // extern "C"

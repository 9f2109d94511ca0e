// An entry point that never allocates device memory.
//
// Who needs it: host code that cannot or must not call cudaMalloc when it
// solves, for example an application that has handed its whole device memory
// budget to its own pool (a further cudaMalloc would fail or fragment that
// pool), or a latency-critical loop that cannot afford the implicit device
// synchronisation an allocation may bring.  Such callers still pass their own
// inputs and output; the only memory the solve needs beyond them -- the
// forward-sweep coefficients of the Thomas recurrence -- lives in a fixed
// array compiled into this library.
//
// Limit: that array holds kNoAllocElems = 2^21 unknowns (two FP32 arrays of
// 2^21 elements, 16 MiB), so num_systems * n must not exceed 2^21.  Every GPU
// that loads the library keeps those 16 MiB until the process exits.
//
// The scratch is shared by every call on a device and keeps whatever the last
// call left in it.  The kernel writes each scratch element before it reads
// it, so nothing has to start at zero.  Calls whose kernels overlap on the
// GPU (different streams, or several host threads) race on the array: issue
// them on one stream or serialise them.
//
// Set-up: the first call on a device looks up the array's device address
// (cudaGetSymbolAddress, with that device current) and caches it; make that
// first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "tridi.h"
#include "tridi_device.cuh"

namespace tridi {
namespace {

constexpr long kNoAllocElems = 1L << 21;

// c' then d' of the forward sweep, kNoAllocElems each.
static __device__ __align__(256) float g_noalloc_scratch[2 * kNoAllocElems];

constexpr int kMaxDev = 64;
float* g_scratch_ptr[kMaxDev] = {};
std::mutex g_scratch_mu;
thread_local int t_noalloc_cuda_error = 0;

// Thomas recurrence of the gold solver (tridiagonal_gold.h:26-44, a[0] and
// c[n-1] taken as zero), one thread per system of an interleaved batch
// (element i of system s at i*m + s), so a warp's row accesses are 128-byte
// lines.  cp and dp point into the static scratch.
__global__ void __launch_bounds__(256) thomas_interleaved_noalloc_kernel(const float* a, const float* b,
                                                                         const float* c, const float* d, float* x,
                                                                         long n, long m, float* cp, float* dp) {
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= m) return;
  float cprev = 0.f, dprev = 0.f;
  for (long i = 0; i < n; ++i) {
    const long k = i * m + s;
    const float ai = i == 0 ? 0.f : a[k];
    const float ci = i == n - 1 ? 0.f : c[k];
    const float inv = tdiv(1.f, b[k] - ai * cprev);
    cprev = ci * inv;
    dprev = (d[k] - ai * dprev) * inv;
    cp[k] = cprev;
    dp[k] = dprev;
  }
  float xn = dprev;
  x[(n - 1) * m + s] = xn;
  for (long i = n - 2; i >= 0; --i) {
    const long k = i * m + s;
    xn = dp[k] - cp[k] * xn;
    x[k] = xn;
  }
}

// Device address of the scratch on the current device, looked up once.
tridi_status scratch_on_current_device(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    t_noalloc_cuda_error = (int)e;
    return TRIDI_ERROR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDev) return TRIDI_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      t_noalloc_cuda_error = (int)(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
      return TRIDI_ERROR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  *out = g_scratch_ptr[dev];
  return TRIDI_SUCCESS;
}

}  // namespace
}  // namespace tridi

extern "C" {

long tridi_noalloc_max_unknowns(void) { return tridi::kNoAllocElems; }

int tridi_noalloc_last_cuda_error(void) { return tridi::t_noalloc_cuda_error; }

tridi_status tridi_solve_interleaved_noalloc_f32(const float* a, const float* b, const float* c, const float* d,
                                                 float* x, long n, long num_systems, tridi_stream_t stream) {
  using namespace tridi;
  if (!a || !b || !c || !d || !x || n <= 0 || num_systems <= 0) return TRIDI_ERROR_INVALID_VALUE;
  if (n > kNoAllocElems / num_systems) return TRIDI_ERROR_WORKSPACE_TOO_SMALL;  // n * m > the static scratch
  float* scratch = nullptr;
  tridi_status st = scratch_on_current_device(&scratch);
  if (st != TRIDI_SUCCESS) return st;
  const unsigned blocks = (unsigned)((num_systems + 255) / 256);
  thomas_interleaved_noalloc_kernel<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      a, b, c, d, x, n, num_systems, scratch, scratch + kNoAllocElems);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    t_noalloc_cuda_error = (int)e;
    return TRIDI_ERROR_CUDA;
  }
  return TRIDI_SUCCESS;
}

}  // extern "C"

// Autotuner: picks, per size (bucket), the launch choices that the public
// entry points otherwise make by fixed rules, by timing every candidate on a
// seeded synthetic batch on the caller's GPU.  No counterpart in the
// reference, whose switch levels and splits are compile-time or caller-given
// constants.
//
//   TRIDI_AUTOTUNE_CRPCR_REST        CR-to-PCR switch level per power-of-two n
//   TRIDI_AUTOTUNE_PCR_THOMAS_SPLIT  PCR/Thomas split (Thomas chains g) per n
//   TRIDI_AUTOTUNE_RAGGED_THREADS    threads per system per size bucket of the
//                                    ragged work queue (32, 160 or 480)
//   TRIDI_AUTOTUNE_CR_ROWS           rows per thread of the FP32 CR / PCR /
//                                    CR-PCR kernels per power-of-two n
//   TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS  threads per system per size bucket
//                                    of plans for the fused refinement, timed
//                                    on that refinement (one correction)
//
// The choices land in the process-wide table of runtime.cu (tridi_tuned /
// tridi_set_tuned); the Python layer saves and reloads it as JSON.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "runtime.h"
#include "tridi.h"

namespace tridi {
namespace {

__device__ __forceinline__ float unit_hash(unsigned long long i, unsigned salt) {
  unsigned h = (unsigned)(i * 0x9E3779B97F4A7C15ULL >> 32) ^ salt;
  h ^= h >> 16;
  h *= 0x7feb352dU;
  h ^= h >> 15;
  h *= 0x846ca68bU;
  h ^= h >> 16;
  return (h >> 8) * (1.0f / 16777216.0f);  // [0, 1)
}

// Diagonally dominant rows (a, c ~ U[-1,1], b = |a|+|c|+U[1,2], d ~ U[-1,1]);
// adi: a = c = -r, b = 1 + 2r with r ~ U[0.1, 10] per row.  Every row gets
// values, so pad rows are defined too.
__global__ void synth_kernel(float* a, float* b, float* c, float* d, long rows, int adi) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const float u1 = unit_hash(i, 0x1234567u), u2 = unit_hash(i, 0x89abcdefu), u3 = unit_hash(i, 0x2468aceu);
  if (adi) {
    const float r = 0.1f + 9.9f * u1;
    a[i] = -r;
    c[i] = -r;
    b[i] = 1.f + 2.f * r;
  } else {
    const float av = 2.f * u1 - 1.f, cv = 2.f * u2 - 1.f;
    a[i] = av;
    c[i] = cv;
    b[i] = fabsf(av) + fabsf(cv) + 1.f + u3;
  }
  d[i] = 2.f * unit_hash(i, 0x5555aaaau) - 1.f;
}

struct Sample {
  float* p = nullptr;
  long rows = 0;
  float *a = nullptr, *b = nullptr, *c = nullptr, *d = nullptr, *x = nullptr;
  ~Sample() {
    if (p) cudaFree(p);
  }
  tridi_status alloc(long r, cudaStream_t st, int adi) {
    rows = (r + 63) & ~63L;
    cudaError_t e = cudaMalloc(&p, sizeof(float) * 5 * rows);
    if (e != cudaSuccess) return cuda_status(e);
    a = p;
    b = a + rows;
    c = b + rows;
    d = c + rows;
    x = d + rows;
    synth_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, st>>>(a, b, c, d, rows, adi);
    return cuda_status(cudaGetLastError());
  }
};

// Milliseconds per call of fn on st: 2 warm-up calls, then the best of 3
// timed groups of 3 (the least disturbed by other work on the GPU).
template <class F>
tridi_status time_ms(F&& fn, cudaStream_t st, float* out) {
  cudaEvent_t e0, e1;
  cudaError_t e;
  if ((e = cudaEventCreate(&e0)) != cudaSuccess) return cuda_status(e);
  if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_status(e);
  }
  tridi_status ts = TRIDI_SUCCESS;
  float best = INFINITY;
  for (int w = 0; w < 2 && ts == TRIDI_SUCCESS; ++w) ts = fn();
  for (int g = 0; g < 3 && ts == TRIDI_SUCCESS; ++g) {
    cudaEventRecord(e0, st);
    for (int r = 0; r < 3 && ts == TRIDI_SUCCESS; ++r) ts = fn();
    cudaEventRecord(e1, st);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
      ts = cuda_status(e);
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = fminf(best, ms / 3.f);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *out = best;
  return ts;
}

}  // namespace
}  // namespace tridi

extern "C" tridi_status tridi_autotune(int table, long key, long sample, tridi_stream_t stream, int* chosen,
                                       float* best_ms) {
  using namespace tridi;
  if (key < 1) return TRIDI_ERROR_INVALID_VALUE;
  if (sample <= 0) sample = 1L << 24;
  cudaStream_t st = as_stream(stream);
  std::vector<int> cands;
  int best = 0;
  float best_t = INFINITY;
  if (table == TRIDI_AUTOTUNE_CRPCR_REST || table == TRIDI_AUTOTUNE_PCR_THOMAS_SPLIT) {
    const int n = (int)key;
    const bool crpcr = table == TRIDI_AUTOTUNE_CRPCR_REST;
    if (!is_pow2(n) || n > 4096 || n < (crpcr ? 4 : 2)) return TRIDI_ERROR_UNSUPPORTED_SIZE;
    const long m = sample / n > 0 ? sample / n : 1;
    Sample smp;
    tridi_status ts = smp.alloc(m * n, st, 0);
    if (ts != TRIDI_SUCCESS) return ts;
    for (int v = crpcr ? 2 : 1; v <= (crpcr ? n / 2 : n); v *= 2) {
      float ms = 0.f;
      ts = time_ms(
          [&]() {
            return crpcr ? tridi_crpcr_f32(smp.a, smp.b, smp.c, smp.d, smp.x, n, (int)m, v, stream)
                         : tridi_pcr_thomas_f32(smp.a, smp.b, smp.c, smp.d, smp.x, n, (int)m, v, stream);
          },
          st, &ms);
      if (ts == TRIDI_ERROR_UNSUPPORTED_SIZE) continue;  // a shape this size does not launch
      if (ts != TRIDI_SUCCESS) return ts;
      if (ms < best_t) {
        best_t = ms;
        best = v;
      }
    }
  } else if (table == TRIDI_AUTOTUNE_CR_ROWS) {
    const int n = (int)key;
    if (!is_pow2(n) || n < 32 || n > 4096) return TRIDI_ERROR_UNSUPPORTED_SIZE;
    const long m = sample / n > 0 ? sample / n : 1;
    Sample smp;
    tridi_status ts = smp.alloc(m * n, st, 0);
    if (ts != TRIDI_SUCCESS) return ts;
    const int saved = tuned(table, ilog2(n));
    for (int rows : {4, 8, 16}) {
      if (n / rows > 256 || n / rows < 2) continue;
      tridi_set_tuned(table, key, rows);
      float ms = 0.f;
      ts = time_ms([&]() { return tridi_cr_f32(smp.a, smp.b, smp.c, smp.d, smp.x, n, (int)m, stream); }, st, &ms);
      if (ts == TRIDI_ERROR_UNSUPPORTED_SIZE) continue;
      if (ts != TRIDI_SUCCESS) break;
      if (ms < best_t) {
        best_t = ms;
        best = rows;
      }
    }
    tridi_set_tuned(table, key, saved);
    if (ts != TRIDI_SUCCESS && ts != TRIDI_ERROR_UNSUPPORTED_SIZE) return ts;
  } else if (table == TRIDI_AUTOTUNE_RAGGED_THREADS || table == TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS) {
    const bool refine = table == TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS;
    const int k = ilog2(key);
    const long lo = 1L << k;
    long hi = (2L << k) - 1;
    if (k > 14) return TRIDI_ERROR_UNSUPPORTED_SIZE;
    if (hi > 24480) hi = 24480;
    // above the team limit every candidate gives a system the whole CTA: time
    // only the sizes the choice decides (for [8192, 16384): 8192 .. ~8950)
    const long cap = ragged_team_max_rows() - 8;
    if (lo <= cap && hi > cap) hi = cap;
    // sizes spread evenly over the bucket, enough systems for `sample` rows
    std::vector<long> off(1, 0);
    for (long s = 0; off.back() < sample && s < (1L << 22); ++s)
      off.push_back(off.back() + lo + (long)((s * 2654435761UL) % (unsigned long)(hi - lo + 1)));
    const int nsys = (int)off.size() - 1;
    Sample smp;
    tridi_status ts = smp.alloc(off.back() + 4, st, 1);
    if (ts != TRIDI_SUCCESS) return ts;
    // the refinement's FP64 solution, workspace and residual word
    const size_t wsb = refine ? tridi_ragged_refine_workspace_bytes(off.back(), nsys) : 0;
    void* rbuf = nullptr;
    if (refine) {
      const cudaError_t e = cudaMalloc(&rbuf, wsb + sizeof(double) * (size_t)(off.back() + 4 + 31 + 32));
      if (e != cudaSuccess) return cuda_status(e);
    }
    double* x64 = static_cast<double*>(rbuf);
    double* rel = x64 + ((off.back() + 4 + 31) & ~31L);
    void* ws = rel + 32;
    const int saved = tuned(table, k);
    for (int th : {32, 160, 480}) {
      tridi_set_tuned(table, key, th);
      void* plan = nullptr;
      ts = refine ? tridi_ragged_plan_create_refine(off.data(), nsys, &plan)
                  : tridi_ragged_plan_create(off.data(), nsys, &plan);
      if (ts != TRIDI_SUCCESS) break;
      const size_t pb = tridi_ragged_plan_device_bytes(plan);
      void* dp = nullptr;
      cudaError_t e = cudaMalloc(&dp, pb);
      if (e != cudaSuccess) {
        tridi_ragged_plan_destroy(plan);
        ts = cuda_status(e);
        break;
      }
      ts = tridi_ragged_plan_upload(plan, dp, pb, stream);
      float ms = 0.f;
      if (ts == TRIDI_SUCCESS)
        ts = time_ms(
            [&]() {
              return refine ? tridi_ragged_refine_f32(smp.a, smp.b, smp.c, smp.d, x64, plan, dp, nullptr, 1, ws, wsb,
                                                      rel, stream)
                            : tridi_ragged_solve_f32(smp.a, smp.b, smp.c, smp.d, smp.x, plan, dp, stream);
            },
            st, &ms);
      cudaFree(dp);
      tridi_ragged_plan_destroy(plan);
      if (ts != TRIDI_SUCCESS) break;
      if (ms < best_t) {
        best_t = ms;
        best = th;
      }
    }
    tridi_set_tuned(table, key, saved);
    if (rbuf) cudaFree(rbuf);
    if (ts != TRIDI_SUCCESS) return ts;
  } else {
    return TRIDI_ERROR_INVALID_VALUE;
  }
  if (best == 0) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  tridi_status ts = tridi_set_tuned(table, key, best);
  if (ts != TRIDI_SUCCESS) return ts;
  if (chosen) *chosen = best;
  if (best_ms) *best_ms = best_t;
  return TRIDI_SUCCESS;
}

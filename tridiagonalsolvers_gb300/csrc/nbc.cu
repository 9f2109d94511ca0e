// Launch logic and C-ABI entry points of the bank-conflict-free CR: the
// register kernels of hybrid.cu and crpcr2.cu by default (the same CR
// arithmetic, results bit-identical to the shared-memory kernel for crNBC,
// within a few ulp for crpcrNBC, about twice its speed), the
// shared-memory CR of nbc.cuh on request (TRIDI_TUNE_NBC_KERNEL = 2) or where
// the register kernel has no shape.  Replaces the device work of crNBC()
// (crNBC.cu:123), crNBC32() (crNBC32banks.cu:123) and crpcrNBC()
// (crNBC.cu:344).
#include "nbc.cuh"
#include "runtime.h"

namespace tridi {

namespace {

constexpr int kMaxThreads = 4 * 32 + 32;

template <class T>
tridi_status solve_nbc(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m, int rest,
                       tridi_stream_t stream) {
  if (!a || !b || !c || !d || !x || m <= 0) return TRIDI_ERROR_INVALID_VALUE;
  const int nmax = sizeof(T) == 4 ? 4096 : 2048;
  if (!is_pow2(n) || n < 2 || n > nmax) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  if (!is_pow2(rest) || rest < 2 || rest > (n > 2 ? n / 2 : 2)) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  if (tunable(TRIDI_TUNE_NBC_KERNEL) != 2) {
    // the register kernels: the same CR arithmetic (bit-identical results at
    // rest 2; the PCR of crpcr's register kernels at 1024 unknowns works on
    // normalised rows, a few ulp apart), no shared-memory bank traffic
    tridi_status st;
    if constexpr (sizeof(T) == 4)
      st = rest == 2 ? tridi_cr_f32(a, b, c, d, x, n, m, stream) : tridi_crpcr_f32(a, b, c, d, x, n, m, rest, stream);
    else
      st = rest == 2 ? tridi_cr_f64(a, b, c, d, x, n, m, stream) : tridi_crpcr_f64(a, b, c, d, x, n, m, rest, stream);
    if (st != TRIDI_ERROR_UNSUPPORTED_SIZE) return st;
  }
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;

  NbcParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.rest = rest;
  p.status = dev->status;
  const bool tma_ok = aligned16(a) && aligned16(b) && aligned16(c) && aligned16(d) &&
                      ((size_t)n * sizeof(T)) % 16 == 0 && !g_host_mapped_io;
  p.vec = aligned16(x) ? 1 : 0;
  const size_t limit = (size_t)dev->max_smem_optin;
  const size_t target = 110 * 1024;  // two CTAs per SM when it fits
  int G = 4, S = 0;
  for (; G >= 1; --G) {
    const size_t fixed = NbcSmem<T>::bytes(0, G, n, rest);
    const size_t stage = (size_t)4 * G * n * sizeof(T);
    if (!tma_ok) {
      if (fixed <= limit) break;
      continue;
    }
    if (fixed + 2 * stage <= target || (G == 1 && fixed + stage <= limit)) {
      S = pick_stages(fixed, stage, 1, *dev);
      break;
    }
  }
  if (G < 1) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  p.G = G;
  p.stages = S;
  p.ntiles = (int)(((long)m + G - 1) / G);
  const size_t smem = NbcSmem<T>::bytes(S, G, n, rest);
  auto kern = nbc_kernel<T, kMaxThreads, sizeof(T) == 4 ? 5 : 1>;  // FP32: 5 CTAs (20 solving warps) per SM
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  const int threads = 32 * G + 32;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem)) != cudaSuccess)
    return cuda_status(e);
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev->sm_count;
  if (grid > p.ntiles) grid = p.ntiles;
  kern<<<(unsigned)grid, threads, smem, as_stream(stream)>>>(p);
  return cuda_status(cudaGetLastError());
}

}  // namespace
}  // namespace tridi

using tridi::solve_nbc;

extern "C" {

tridi_status tridi_cr_nbc_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                              int m, tridi_stream_t s) {
  return solve_nbc<float>(a, b, c, d, x, n, m, 2, s);
}
tridi_status tridi_cr_nbc_f64(const double* a, const double* b, const double* c, const double* d, double* x,
                              int n, int m, tridi_stream_t s) {
  return solve_nbc<double>(a, b, c, d, x, n, m, 2, s);
}
tridi_status tridi_crpcr_nbc_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                                 int m, int rest, tridi_stream_t s) {
  if (n < 4) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  return solve_nbc<float>(a, b, c, d, x, n, m, rest, s);
}
tridi_status tridi_crpcr_nbc_f64(const double* a, const double* b, const double* c, const double* d, double* x,
                                 int n, int m, int rest, tridi_stream_t s) {
  if (n < 4) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  return solve_nbc<double>(a, b, c, d, x, n, m, rest, s);
}

}  // extern "C"

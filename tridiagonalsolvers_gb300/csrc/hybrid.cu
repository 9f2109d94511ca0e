// Launch logic and C-ABI entry points of the CR / PCR / hybrid family
// (hybrid.cuh).  Replaces the device work of cr() (cr_app.cu:4), pcr()
// (pcr_app.cu:5) and crpcr() (crpcr_app.cu:5).
#include "hybrid.cuh"
#include "pcr_twophase.cuh"
#include "runtime.h"

namespace tridi {

namespace {

// Per-(precision, n) shape: K rows per thread, TPS = n/K threads per system.
// Groups of at most one warp use shuffles; wider groups use shared memory.
struct Shape {
  int K;
  int tps;
  bool warp;
};

template <class T>
bool choose_shape(int n, Shape* s) {
  if (!is_pow2(n) || n < 2) return false;
  int K;
  if (sizeof(T) == 4) {
    if (n > 4096) return false;
    K = n <= 16 ? n / 2 : (n == 4096 ? 16 : 8);
  } else {
    if (n > 2048) return false;
    K = n <= 8 ? n / 2 : (n == 2048 ? 8 : 4);
  }
  // rows per thread: the process-wide tunable, else the autotuned choice for
  // this n (FP32 only), else the rule above
  int tk = tunable(TRIDI_TUNE_CR_ROWS);
  if (tk <= 0 && sizeof(T) == 4) tk = tuned(TRIDI_AUTOTUNE_CR_ROWS, ilog2(n));
  if (tk > 0 && is_pow2(tk) && tk <= n / 2 && n / tk <= 256) {
    // only shapes with an instantiated kernel (see solve_hybrid)
    const bool warp = n / tk <= 32;
    const bool have = sizeof(T) == 4 ? (warp ? tk <= 16 : (tk == 8 || tk == 16)) : (warp ? tk <= 4 : (tk == 4 || tk == 8));
    if (have) K = tk;
  }
  s->K = K;
  s->tps = n / K;
  s->warp = s->tps <= 32;
  return true;
}

constexpr int kWarpThreads = 128 + 32;   // 4 consumer warps + producer warp
constexpr int kBlockThreads = 256 + 32;  // up to 8 consumer warps + producer

// Warp shapes with bulk-copy alignment: hybrid_warp_kernel, two buffers per
// warp, as many CTAs of 4 warps as registers and shared memory allow.
template <class T, int K, int LSTRIDE>
cudaError_t launch_warp_streams(const HybridParams& p, const DeviceInfo& dev, cudaStream_t stream) {
  constexpr int MINB = K >= 16 ? 4 : 5;  // 5: at most 96 registers, 20 warps per SM
  auto kern = hybrid_warp_kernel<T, K, LSTRIDE, MINB>;
  const int warps = kWarpKernelThreads / 32;
  const size_t smem = HybridSmem<T>::barrier_bytes() + (size_t)warps * 2 * HybridSmem<T>::stage_elems(32 / p.tps, p.n) * sizeof(T);
  if (smem > (size_t)dev.max_smem_optin) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarpKernelThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const long tiles = ((long)p.m + 32 / p.tps - 1) / (32 / p.tps);
  long grid = (long)per_sm * dev.sm_count;
  if (grid * warps > tiles) grid = (tiles + warps - 1) / warps;
  kern<<<(unsigned)grid, kWarpKernelThreads, smem, stream>>>(p);
  return cudaGetLastError();
}

// Block shapes with one 128-thread CTA of groups (tps 64 or 128) and
// bulk-copy alignment: hybrid_block_stream_kernel, no producer warp.
template <class T, int K, int LSTRIDE>
cudaError_t launch_block_streams(const HybridParams& p, const DeviceInfo& dev, cudaStream_t stream) {
  constexpr int MINB = K >= 16 ? 4 : 5;
  auto kern = hybrid_block_stream_kernel<T, K, LSTRIDE, 128, MINB>;
  const size_t smem = HybridSmem<T>::bytes(2, p.G, p.n, p.scratch_rows, false, p.ct, Log2<K>::value);
  if (smem > (size_t)dev.max_smem_optin) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, p.ct, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev.sm_count;
  if (grid > p.ntiles) grid = p.ntiles;
  kern<<<(unsigned)grid, p.ct, smem, stream>>>(p);
  return cudaGetLastError();
}

template <class T, int K, bool WARP, int LSTRIDE>
cudaError_t launch_one(const HybridParams& p0, const DeviceInfo& dev, cudaStream_t stream) {
  constexpr int MAXT = WARP ? kWarpThreads : kBlockThreads;
  constexpr int MINB = WARP ? 3 : 2;
  auto kern = hybrid_kernel<T, K, WARP, LSTRIDE, MAXT, MINB>;
  HybridParams p = p0;
  const bool tma_ok = aligned16(p.a) && aligned16(p.b) && aligned16(p.c) && aligned16(p.d) && aligned16(p.x) &&
                      ((size_t)p.n * sizeof(T)) % 16 == 0 && !g_host_mapped_io;
  // (FP32 shapes that keep their registers at 20 warps per SM; the FP64
  // shapes and PCR on 16 rows per thread would spill)
  if constexpr (WARP && sizeof(T) == 4 && !(K == 16 && LSTRIDE == 1)) {
    if (tma_ok && tunable(TRIDI_TUNE_WARP_STREAMS) != 2) return launch_warp_streams<T, K, LSTRIDE>(p, dev, stream);
  }
  if constexpr (!WARP && sizeof(T) == 4 && !(K == 16 && LSTRIDE == 1)) {
    if (tma_ok && p.ct == 128 && tunable(TRIDI_TUNE_WARP_STREAMS) != 2)
      return launch_block_streams<T, K, LSTRIDE>(p, dev, stream);
  }
  const int logk = Log2<K>::value;
  const size_t stage_bytes = HybridSmem<T>::stage_elems(p.G, p.n) * sizeof(T);
  const size_t fixed = HybridSmem<T>::bytes(0, p.G, p.n, p.scratch_rows, WARP, p.ct, logk);
  const int S = tma_ok ? pick_stages(fixed, stage_bytes, 2, dev) : 0;
  p.stages = S;
  const size_t smem = HybridSmem<T>::bytes(S, p.G, p.n, p.scratch_rows, WARP, p.ct, logk);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int threads = p.ct + 32;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev.sm_count;
  if (grid > p.ntiles) grid = p.ntiles;
  kern<<<(unsigned)grid, threads, smem, stream>>>(p);
  return cudaGetLastError();
}

// FP32 PCR on 64..1024 unknowns: the two-phase kernel (pcr_twophase.cuh).
// Each array is a tensor of rows of 32 values; a warp tile is a box of R
// such rows.
template <int N, bool PAIRED>
cudaError_t launch_pcr_twophase(const HybridParams& p, const DeviceInfo& dev, cudaStream_t stream) {
  using S = Pcr2Shape<N>;
  auto kern = pcr_twophase_kernel<N, PAIRED>;
  constexpr int kThreads = S::WARPS * 32;
  const uint64_t rows = (uint64_t)p.m * N / 32;
  CUtensorMap ma, mb, mc, md;
  if (!make_tensor_map_2d(&ma, static_cast<const float*>(p.a), 32, rows, 128, 32, S::R, true) ||
      !make_tensor_map_2d(&mb, static_cast<const float*>(p.b), 32, rows, 128, 32, S::R, true) ||
      !make_tensor_map_2d(&mc, static_cast<const float*>(p.c), 32, rows, 128, 32, S::R, true) ||
      !make_tensor_map_2d(&md, static_cast<const float*>(p.d), 32, rows, 128, 32, S::R, true))
    return cudaErrorInvalidValue;
  if (S::SMEM > (size_t)dev.max_smem_optin) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, S::SMEM);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const long tiles = ((long)p.m + S::SPW - 1) / S::SPW;
  long grid = (long)per_sm * dev.sm_count;
  if (grid * S::WARPS > tiles) grid = (tiles + S::WARPS - 1) / S::WARPS;
  kern<<<(unsigned)grid, kThreads, S::SMEM, stream>>>(p, ma, mb, mc, md);
  return cudaGetLastError();
}

template <class T>
bool pcr_twophase_applies(const HybridParams& p) {
  if constexpr (sizeof(T) != 4) return false;
  return p.stride == 1 && (p.n == 64 || p.n == 128 || p.n == 256 || p.n == 512 || p.n == 1024) && aligned16(p.a) &&
         aligned16(p.b) && aligned16(p.c) && aligned16(p.d) && (long)p.m * p.n / 32 < (1L << 31) &&
         tunable(TRIDI_TUNE_PCR_KERNEL) != 2 && !g_host_mapped_io;
}

template <class T>
tridi_status solve_hybrid(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m, int stride,
                          tridi_stream_t stream) {
  if (!a || !b || !c || !d || !x || m <= 0) return TRIDI_ERROR_INVALID_VALUE;
  Shape sh;
  if (!choose_shape<T>(n, &sh)) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  HybridParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.tps = sh.tps; p.stride = stride;
  p.ct = sh.warp ? 128 : (sh.tps > 128 ? sh.tps : 128);
  p.G = p.ct / sh.tps;
  p.scratch_rows = stride < sh.K ? n / stride : sh.tps;
  p.ntiles = (int)(((long)m + p.G - 1) / p.G);
  p.status = dev->status;
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaErrorInvalidValue;
  if constexpr (sizeof(T) == 4) {
    if (crpcr_regs_applies(a, b, c, d, x, n, m, stride)) return crpcr_regs_solve(a, b, c, d, x, n, m, stride, s);
    if (pcr_twophase_applies<T>(p)) {
      const bool paired = tunable(TRIDI_TUNE_PCR_KERNEL) != 3;
      switch (n) {
        case 64: return cuda_status(paired ? launch_pcr_twophase<64, true>(p, *dev, s)
                                           : launch_pcr_twophase<64, false>(p, *dev, s));
        case 128: return cuda_status(paired ? launch_pcr_twophase<128, true>(p, *dev, s)
                                            : launch_pcr_twophase<128, false>(p, *dev, s));
        case 256: return cuda_status(paired ? launch_pcr_twophase<256, true>(p, *dev, s)
                                            : launch_pcr_twophase<256, false>(p, *dev, s));
        case 512: return cuda_status(paired ? launch_pcr_twophase<512, true>(p, *dev, s)
                                            : launch_pcr_twophase<512, false>(p, *dev, s));
        default: return cuda_status(paired ? launch_pcr_twophase<1024, true>(p, *dev, s)
                                           : launch_pcr_twophase<1024, false>(p, *dev, s));
      }
    }
  }
  const int ls = stride < sh.K ? stride : 0;
#define TRIDI_LAUNCH_LS(KK, WW, LS) \
  if (sh.K == KK && sh.warp == WW && ls == LS) e = launch_one<T, KK, WW, LS>(p, *dev, s);
#define TRIDI_LAUNCH(KK, WW)                                                             \
  TRIDI_LAUNCH_LS(KK, WW, 0)                                                              \
  if constexpr (KK > 1) { TRIDI_LAUNCH_LS(KK, WW, 1) }                                    \
  if constexpr (KK > 2) { TRIDI_LAUNCH_LS(KK, WW, (KK > 2 ? 2 : 1)) }                     \
  if constexpr (KK > 4) { TRIDI_LAUNCH_LS(KK, WW, (KK > 4 ? 4 : 1)) }                     \
  if constexpr (KK > 8) { TRIDI_LAUNCH_LS(KK, WW, (KK > 8 ? 8 : 1)) }
  if constexpr (sizeof(T) == 4) {
    TRIDI_LAUNCH(1, true) TRIDI_LAUNCH(2, true) TRIDI_LAUNCH(4, true) TRIDI_LAUNCH(8, true)
    TRIDI_LAUNCH(16, true) TRIDI_LAUNCH(8, false) TRIDI_LAUNCH(16, false)
  } else {
    TRIDI_LAUNCH(1, true) TRIDI_LAUNCH(2, true) TRIDI_LAUNCH(4, true) TRIDI_LAUNCH(4, false)
    TRIDI_LAUNCH(8, false)
  }
#undef TRIDI_LAUNCH
#undef TRIDI_LAUNCH_LS
  return cuda_status(e);
}

}  // namespace

// Exposed to the other translation units (refinement, drop-ins).
template <class T>
tridi_status hybrid_solve_device(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m, int stride,
                                 tridi_stream_t stream) {
  return solve_hybrid<T>(a, b, c, d, x, n, m, stride, stream);
}
template tridi_status hybrid_solve_device<float>(const float*, const float*, const float*, const float*, float*,
                                                 int, int, int, tridi_stream_t);
template tridi_status hybrid_solve_device<double>(const double*, const double*, const double*, const double*,
                                                  double*, int, int, int, tridi_stream_t);

}  // namespace tridi

using tridi::solve_hybrid;

namespace {
template <class T>
tridi_status crpcr_checked(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m, int rest,
                           tridi_stream_t s) {
  if (n < 4 || !tridi::is_pow2(rest) || rest < 2 || rest > n / 2 || !tridi::is_pow2(n))
    return TRIDI_ERROR_UNSUPPORTED_SIZE;
  return solve_hybrid<T>(a, b, c, d, x, n, m, n / rest, s);
}
}  // namespace

extern "C" {

tridi_status tridi_cr_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n, int m,
                          tridi_stream_t s) {
  return solve_hybrid<float>(a, b, c, d, x, n, m, n / 2 > 0 ? n / 2 : 1, s);
}
tridi_status tridi_cr_f64(const double* a, const double* b, const double* c, const double* d, double* x, int n,
                          int m, tridi_stream_t s) {
  return solve_hybrid<double>(a, b, c, d, x, n, m, n / 2 > 0 ? n / 2 : 1, s);
}
tridi_status tridi_pcr_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n, int m,
                           tridi_stream_t s) {
  if (n > 4096) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  return solve_hybrid<float>(a, b, c, d, x, n, m, 1, s);
}
tridi_status tridi_pcr_f64(const double* a, const double* b, const double* c, const double* d, double* x, int n,
                           int m, tridi_stream_t s) {
  return solve_hybrid<double>(a, b, c, d, x, n, m, 1, s);
}
tridi_status tridi_crpcr_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                             int m, int rest, tridi_stream_t s) {
  return crpcr_checked<float>(a, b, c, d, x, n, m, rest, s);
}
tridi_status tridi_crpcr_f64(const double* a, const double* b, const double* c, const double* d, double* x,
                             int n, int m, int rest, tridi_stream_t s) {
  return crpcr_checked<double>(a, b, c, d, x, n, m, rest, s);
}

}  // extern "C"

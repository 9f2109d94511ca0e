// Uniform-size batched partition solve (partition.cuh): tridi_solve_*.
// Warp mode: one warp per system (n <= 32*K), G = 4 systems per tile.
// CTA mode: one CTA of ct threads per system; the ct separators form a
// second tridiagonal system, solved by PCR across the CTA in shared memory.
// Inputs arrive through the cp.async.bulk + mbarrier ring of hybrid.cuh.
#include "partition.cuh"
#include "runtime.h"

namespace tridi {

struct PartParams {
  const void* a;
  const void* b;
  const void* c;
  const void* d;
  void* x;
  int n, m;
  int G;       // systems per tile
  int ntiles;
  int stages;  // 0: read rows straight from global memory
  int kk;      // rows per lane (odd)
  int ct;      // consumer threads
  unsigned* status;
};

template <class T>
__host__ __device__ inline size_t part_smem_bytes(int stages, int G, int n, int ct, bool cta) {
  size_t s = 128 + (size_t)stages * 4 * G * n * sizeof(T);
  if (cta) s += ((size_t)ct * 5 + (size_t)(ct / 32) * 3) * sizeof(T);
  return s;
}

template <class T, int K, bool CTA, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) partition_kernel(PartParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + 8;
  const int S = p.stages, n = p.n, G = p.G, ct = p.ct, kk = p.kk;
  T* stages = reinterpret_cast<T*>(smem + 128);
  const size_t stage_elems = (size_t)4 * G * n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0 && S > 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], ct / 32);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const T* ga = static_cast<const T*>(p.a);
  const T* gb = static_cast<const T*>(p.b);
  const T* gc = static_cast<const T*>(p.c);
  const T* gd = static_cast<const T*>(p.d);
  T* gx = static_cast<T*>(p.x);

  if (tid >= ct) {  // producer warp
    if (S > 0 && lane == 0) {
      int k = 0;
      for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
        const int s = k % S;
        if (k >= S && !mbar_wait(&empty[s], ((k / S) - 1) & 1, p.status)) break;
        const long sys0 = (long)tile * G;
        const long nsys = (p.m - sys0) < G ? (p.m - sys0) : G;
        const uint32_t bytes = (uint32_t)(nsys * n * sizeof(T));
        T* st = stages + s * stage_elems;
        mbar_arrive_expect_tx(&full[s], 4 * bytes);
        bulk_g2s(st + 0 * (size_t)G * n, ga + sys0 * n, bytes, &full[s]);
        bulk_g2s(st + 1 * (size_t)G * n, gb + sys0 * n, bytes, &full[s]);
        bulk_g2s(st + 2 * (size_t)G * n, gc + sys0 * n, bytes, &full[s]);
        bulk_g2s(st + 3 * (size_t)G * n, gd + sys0 * n, bytes, &full[s]);
      }
    }
    return;
  }

  // CTA-mode scratch: separator rows R (4 ct), their solution Xs (ct), and
  // each warp's lane-0 first-row coefficients (3 per warp).
  T* Ra = stages + (size_t)S * stage_elems;
  T* Rb = Ra + ct;
  T* Rc = Rb + ct;
  T* Rd = Rc + ct;
  T* Xs = Rd + ct;
  T* F0 = Xs + ct;

  const int g = CTA ? 0 : warp;  // system within the tile
  int k = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
    const long sys = (long)tile * G + g;
    const T *sa, *sb, *sc, *sd;
    int s = 0;
    if (S > 0) {
      s = k % S;
      bool ok = mbar_wait(&full[s], (k / S) & 1, p.status);
      if constexpr (CTA) ok = consumer_sync_and(ct, ok);
      if (!ok) break;
      const T* st = stages + s * stage_elems + (size_t)g * n;
      sa = st; sb = st + (size_t)G * n; sc = st + 2 * (size_t)G * n; sd = st + 3 * (size_t)G * n;
    } else {
      const long sc0 = (sys < p.m ? sys : p.m - 1) * (long)n;
      sa = ga + sc0; sb = gb + sc0; sc = gc + sc0; sd = gd + sc0;
    }
    T x[K];
    int kl = 0;
    int r0;
    if constexpr (!CTA) {
      r0 = lane * kk;
      kl = warp_partition_solve<T, K>(n, kk, sa, sb, sc, sd, x);
    } else {
      r0 = tid * kk;
      int kr = n - r0;
      kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
      kl = kr;
      Chunk<T, K> ch;
      chunk_eliminate<T, K>(ch, kr, tid == 0, r0 + kr == n && kr > 0, sa + r0, sb + r0, sc + r0, sd + r0);
      if (lane == 0) {
        F0[warp * 3 + 0] = ch.fD; F0[warp * 3 + 1] = ch.fC; F0[warp * 3 + 2] = ch.fA;
      }
      consumer_sync(ct);
      T nD = __shfl_down_sync(kFull, ch.fD, 1);
      T nC = __shfl_down_sync(kFull, ch.fC, 1);
      T nA = __shfl_down_sync(kFull, ch.fA, 1);
      if (lane == 31 && warp + 1 < ct / 32) {
        nD = F0[(warp + 1) * 3 + 0]; nC = F0[(warp + 1) * 3 + 1]; nA = F0[(warp + 1) * 3 + 2];
      }
      // The ct separators form a tridiagonal system: PCR across the CTA in
      // shared memory, one row per thread, identity rows past either end.
      Row<T> sr = separator_row<T, K>(ch, nD, nC, nA);
      const Row<T> id{T(0), T(1), T(0), T(0)};
      for (int dl = 1; dl < ct; dl *= 2) {
        Ra[tid] = sr.a; Rb[tid] = sr.b; Rc[tid] = sr.c; Rd[tid] = sr.d;
        consumer_sync(ct);
        const Row<T> L = tid >= dl ? Row<T>{Ra[tid - dl], Rb[tid - dl], Rc[tid - dl], Rd[tid - dl]} : id;
        const Row<T> R = tid + dl < ct ? Row<T>{Ra[tid + dl], Rb[tid + dl], Rc[tid + dl], Rd[tid + dl]} : id;
        sr = reduce_row(sr, L, R);
        consumer_sync(ct);
      }
      Xs[tid] = tdiv(sr.d, sr.b);
      consumer_sync(ct);
      const T sj = Xs[tid];
      const T sl = tid > 0 ? Xs[tid - 1] : T(0);
      chunk_back<T, K>(ch, kr, sj, sl, x);
    }
    if (S > 0) {
      release_stage(&empty[s]);
    }
    if (sys < p.m) {
      T* dst = gx + sys * (long)n + r0;
#pragma unroll
      for (int i = 0; i < K; ++i)
        if (i < kl) dst[i] = x[i];
    }
    if constexpr (CTA) consumer_sync(ct);  // Xs / F0 reused by the next tile
  }
}

namespace {

template <class T, int K, bool CTA>
cudaError_t launch_part(PartParams p, const DeviceInfo& dev, cudaStream_t stream) {
  constexpr int MAXT = CTA ? 512 + 32 : 128 + 32;
  constexpr int MINB = CTA ? 1 : 4;
  auto kern = partition_kernel<T, K, CTA, MAXT, MINB>;
  const bool tma_ok = aligned16(p.a) && aligned16(p.b) && aligned16(p.c) && aligned16(p.d) &&
                      ((size_t)p.n * sizeof(T)) % 16 == 0 && !g_host_mapped_io;
  const size_t stage = (size_t)4 * p.G * p.n * sizeof(T);
  const size_t fixed = part_smem_bytes<T>(0, p.G, p.n, p.ct, CTA);
  const int S = tma_ok ? pick_stages(fixed, stage, 2, dev) : 0;
  p.stages = S;
  const size_t smem = part_smem_bytes<T>(S, p.G, p.n, p.ct, CTA);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, p.ct + 32, smem)) != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev.sm_count;
  if (grid > p.ntiles) grid = p.ntiles;
  kern<<<(unsigned)grid, p.ct + 32, smem, stream>>>(p);
  return cudaGetLastError();
}

int odd_ceil(int v) { return (v % 2) ? v : v + 1; }

}  // namespace

template <class T>
tridi_status partition_solve_device(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m,
                                    tridi_stream_t stream) {
  constexpr bool F32 = sizeof(T) == 4;
  constexpr int kWarpMax = F32 ? 31 : 15;  // rows per lane in warp mode
  constexpr int kCtaMax = F32 ? 17 : 9;    // rows per thread in CTA mode (512 threads)
  if (!a || !b || !c || !d || !x || m <= 0) return TRIDI_ERROR_INVALID_VALUE;
  static_assert(512L * kCtaMax == partition_max_rows<T>(), "partition size cap");
  if (n < 1 || n > partition_max_rows<T>()) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  PartParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.status = dev->status;
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  if (n <= 32 * kWarpMax) {
    p.kk = odd_ceil((n + 31) / 32);
    p.ct = 128;
    p.G = 4;
    p.ntiles = (int)(((long)m + 3) / 4);
    if (p.kk <= 3) e = launch_part<T, 3, false>(p, *dev, s);
    else if (p.kk <= 7) e = launch_part<T, 7, false>(p, *dev, s);
    else if (p.kk <= 9) e = launch_part<T, 9, false>(p, *dev, s);
    else if (p.kk <= 15) e = launch_part<T, 15, false>(p, *dev, s);
    else e = launch_part<T, (F32 ? 31 : 15), false>(p, *dev, s);
  } else {
    int ct = 128;
    while (ct < 512 && odd_ceil((n + ct - 1) / ct) > 7) ct *= 2;
    p.ct = ct;
    p.kk = odd_ceil((n + ct - 1) / ct);
    p.G = 1;
    p.ntiles = m;
    if (p.kk <= 7) e = launch_part<T, 7, true>(p, *dev, s);
    else e = launch_part<T, kCtaMax, true>(p, *dev, s);
  }
  return cuda_status(e);
}

template tridi_status partition_solve_device<float>(const float*, const float*, const float*, const float*, float*,
                                                    int, int, tridi_stream_t);
template tridi_status partition_solve_device<double>(const double*, const double*, const double*, const double*,
                                                     double*, int, int, tridi_stream_t);

}  // namespace tridi

extern "C" {

tridi_status tridi_solve_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n, int m,
                             tridi_stream_t s) {
  return tridi::partition_solve_device<float>(a, b, c, d, x, n, m, s);
}
tridi_status tridi_solve_f64(const double* a, const double* b, const double* c, const double* d, double* x, int n,
                             int m, tridi_stream_t s) {
  return tridi::partition_solve_device<double>(a, b, c, d, x, n, m, s);
}

}  // extern "C"

// PCR-then-Thomas ("pcrGauss", pcrGauss_kernel.cu / pcrGauss_app.cu) on
// sm_103a, exact for every gaussian g.
//
// The reference runs `it` PCR steps and then g strided Thomas chains, with
// (g, it) from fixed tables (pcrGauss_app.cu:12-47, :58-96) in which it is
// often smaller than log2(g): after it steps row i couples to i +- 2^it, so
// chains of stride g > 2^it are not independent and the result is an
// approximation.  Here it = log2(g) always: after log2(g) PCR steps every
// row couples only to rows +-g away, the g chains t, t+g, t+2g, ... are
// independent tridiagonal systems, and Thomas on each is exact.
//
// One system per group of TPS threads, staged into shared memory by the
// cp.async.bulk ring.  PCR: thread t updates rows t, t+TPS, ... (unit stride
// across the warp: conflict-free), all new rows are computed before any is
// written.  Thomas: thread c < g walks chain c (consecutive threads touch
// consecutive rows).  The PCR arithmetic is reduce_row (pcrGauss_kernel.cu:
// 86-98); the Thomas recurrences are those of serial<T,g>
// (pcrGauss_kernel.cu:1-32), except that the last equation's c is ignored
// (the gold solver zeroes it, tridiagonal_gold.h:28).
#include "runtime.h"
#include "tridi_device.cuh"

namespace tridi {

struct PTParams {
  const void* a;
  const void* b;
  const void* c;
  const void* d;
  void* x;
  int n, m;
  int g;        // number of Thomas chains (power of two, 1 <= g <= n)
  int steps;    // log2(g)
  int tps;      // threads per system
  int G;        // systems per tile
  int ntiles;
  int stages;   // >= 1 (bulk copies) or 0 (rows read from global into the work copy)
  int ct;
  unsigned* status;
};

// PCR rows per thread kept in registers between the read and write phases
// (at most; ROWS, the kernel's template argument, is the launch's bound).
constexpr int kPTMaxRows = 16;

template <class T, int MAXT, int ROWS>
__global__ void __launch_bounds__(MAXT) pcr_thomas_kernel(PTParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + 8;
  const int S = p.stages, n = p.n, G = p.G, tps = p.tps, ct = p.ct;
  const size_t stage_elems = (size_t)4 * G * n;
  T* stages = reinterpret_cast<T*>(smem + 128);
  // Work copy of the tile (PCR runs in place here, so the stage can be
  // released as soon as it has been copied).
  T* work = stages + (size_t)(S > 0 ? S : 0) * stage_elems;
  const int tid = threadIdx.x;

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

  if (tid >= ct) {
    if (S > 0 && (tid & 31) == 0) {
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

  const int grp = tid / tps, t = tid - grp * tps;
  T* wa = work + (size_t)grp * n;
  T* wb = wa + (size_t)G * n;
  T* wc = wb + (size_t)G * n;
  T* wd = wc + (size_t)G * n;
  const int rows = (n + tps - 1) / tps;  // rows per thread in the PCR phase

  int k = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
    const long sys = (long)tile * G + grp;
    const long src_sys = sys < p.m ? sys : p.m - 1;
    if (S > 0) {
      const int s = k % S;
      if (!consumer_sync_and(ct, mbar_wait(&full[s], (k / S) & 1, p.status))) break;
      const T* st = stages + s * stage_elems + (size_t)grp * n;
      // the gold solver ignores a[0] and c[n-1]: they are zeroed in the copy
      for (int i = t; i < n; i += tps) {
        wa[i] = i == 0 ? T(0) : st[i];
        wb[i] = st[(size_t)G * n + i];
        wc[i] = i == n - 1 ? T(0) : st[2 * (size_t)G * n + i];
        wd[i] = st[3 * (size_t)G * n + i];
      }
      release_stage(&empty[s]);
    } else {
      for (int i = t; i < n; i += tps) {
        wa[i] = i == 0 ? T(0) : ga[src_sys * n + i];
        wb[i] = gb[src_sys * n + i];
        wc[i] = i == n - 1 ? T(0) : gc[src_sys * n + i];
        wd[i] = gd[src_sys * n + i];
      }
    }
    consumer_sync(ct);

    // ---- log2(g) PCR steps, delta = 1, 2, ..., g/2 ----
    for (int dl = 1; dl < p.g; dl *= 2) {
      Row<T> nr[ROWS];
#pragma unroll
      for (int q = 0; q < ROWS; ++q) {
        const int i = t + q * tps;
        if (q < rows && i < n) {
          const int il = i - dl < 0 ? 0 : i - dl;
          const int ir = i + dl > n - 1 ? n - 1 : i + dl;
          nr[q] = reduce_row(Row<T>{wa[i], wb[i], wc[i], wd[i]}, Row<T>{wa[il], wb[il], wc[il], wd[il]},
                             Row<T>{wa[ir], wb[ir], wc[ir], wd[ir]});
        }
      }
      consumer_sync(ct);
#pragma unroll
      for (int q = 0; q < ROWS; ++q) {
        const int i = t + q * tps;
        if (q < rows && i < n) {
          wa[i] = nr[q].a; wb[i] = nr[q].b; wc[i] = nr[q].c; wd[i] = nr[q].d;
        }
      }
      consumer_sync(ct);
    }

    // ---- g independent Thomas chains of stride g (serial<T,g>) ----
    // (the previous row's c' and d' carried in registers, so each step's
    // dependent chain is arithmetic only; the row loads do not depend on it)
    for (int ch = t; ch < p.g; ch += tps) {
      const int gg = p.g;
      T* __restrict__ cc = wc;
      T* __restrict__ dd = wd;
      const T* __restrict__ aa = wa;
      const T* __restrict__ bb = wb;
      T cprev = tdiv(cc[ch], bb[ch]);
      T dprev = tdiv(dd[ch], bb[ch]);
      cc[ch] = cprev;
      dd[ch] = dprev;
      int last = ch;
      for (int i = ch + gg; i < n; i += gg) {
        const T a = aa[i];
        const T den = bb[i] - a * cprev;
        cprev = tdiv(cc[i], den);
        dprev = tdiv(dd[i] - dprev * a, den);
        cc[i] = cprev;
        dd[i] = dprev;
        last = i;
      }
      T xn = dprev;
      for (int i = last - gg; i >= 0; i -= gg) {
        xn = dd[i] - cc[i] * xn;
        dd[i] = xn;
      }
    }
    consumer_sync(ct);
    if (sys < p.m)
      for (int i = t; i < n; i += tps) gx[sys * n + i] = wd[i];
    consumer_sync(ct);
  }
}

template <class T>
tridi_status hybrid_solve_device(const T*, const T*, const T*, const T*, T*, int, int, int, tridi_stream_t);

namespace {
template <class T>
size_t pt_smem(int S, int G, int n) {
  return 128 + (size_t)S * 4 * G * n * sizeof(T) + (size_t)4 * G * n * sizeof(T);
}
}  // namespace

template <class T>
tridi_status pcr_thomas_device(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m, int g,
                               tridi_stream_t stream) {
  if (!a || !b || !c || !d || !x || m <= 0) return TRIDI_ERROR_INVALID_VALUE;
  const int nmax = 4096;
  if (n < 1 || n > nmax || g < 0) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  const bool pcr_shape = is_pow2(n) && n >= 4 && n <= (sizeof(T) == 4 ? 4096 : 2048);
  if (g == 0) {  // the autotuned split for this n, else n/2 (power-of-two n), else one chain per thread
    const int t = is_pow2(n) ? tuned(TRIDI_AUTOTUNE_PCR_THOMAS_SPLIT, ilog2(n)) : 0;
    if (t > 0 && is_pow2(t) && t <= n) {
      g = t;
    } else if (pcr_shape) {
      g = n / 2;
    } else {
      int tp = 32;
      while (tp < 256 && tp < n) tp *= 2;
      g = 1;
      while (2 * g <= n && 2 * g <= tp) g *= 2;
    }
  }
  if (!is_pow2(g) || g > n) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  // g >= n/2: after log2(n/2) PCR steps the chains are the 2-row systems
  // (j, j + n/2) that close PCR (g = n: one more step decouples every row,
  // the same solution), so the register PCR kernels solve it.
  if (pcr_shape && g >= n / 2) return hybrid_solve_device<T>(a, b, c, d, x, n, m, 1, stream);
  // FP32, 64 .. 1024 unknowns: the register kernel on the two-phase PCR layout
  if constexpr (sizeof(T) == 4) {
    if (pcr_thomas2_applies(a, b, c, d, n, m, g)) return pcr_thomas2_solve(a, b, c, d, x, n, m, g, as_stream(stream));
  }
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  PTParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.g = g; p.status = dev->status;
  int steps = 0;
  while ((1 << steps) < g) ++steps;
  p.steps = steps;
  // threads per system: every PCR row of a thread stays in registers between
  // the read and write phases; up to 4 rows a thread (8, 16 at n = 2048,
  // 4096), so small systems take one or two warps and a CTA holds several
  // systems, whose steps share its barriers, with two CTAs per SM.
  int tps = 32;
  while (tps < 256 && tps * 4 < n) tps *= 2;
  p.tps = tps;
  const int rows = (n + tps - 1) / tps;
  if (rows > kPTMaxRows) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  p.G = 256 / tps > 0 ? 256 / tps : 1;
  while (p.G > 1 && (long)p.G * n * 4 * sizeof(T) > 64 * 1024) p.G /= 2;
  p.ct = p.G * tps;
  p.ntiles = (int)(((long)m + p.G - 1) / p.G);
  const bool tma_ok = aligned16(a) && aligned16(b) && aligned16(c) && aligned16(d) &&
                      ((size_t)n * sizeof(T)) % 16 == 0 && !g_host_mapped_io;
  int S = tma_ok ? 2 : 0;
  while (S > 0 && pt_smem<T>(S, p.G, n) > (size_t)dev->max_smem_optin) --S;
  if (pt_smem<T>(S, p.G, n) > (size_t)dev->max_smem_optin) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  p.stages = S;
  const size_t smem = pt_smem<T>(S, p.G, n);
  auto kern = rows <= 1 ? pcr_thomas_kernel<T, 288, 1>
              : rows <= 2 ? pcr_thomas_kernel<T, 288, 2>
              : rows <= 4 ? pcr_thomas_kernel<T, 288, 4>
              : rows <= 8 ? pcr_thomas_kernel<T, 288, 8>
                          : pcr_thomas_kernel<T, 288, 16>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, p.ct + 32, smem)) != cudaSuccess)
    return cuda_status(e);
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev->sm_count;
  if (grid > p.ntiles) grid = p.ntiles;
  kern<<<(unsigned)grid, p.ct + 32, smem, as_stream(stream)>>>(p);
  return cuda_status(cudaGetLastError());
}

template tridi_status pcr_thomas_device<float>(const float*, const float*, const float*, const float*, float*, int,
                                               int, int, tridi_stream_t);
template tridi_status pcr_thomas_device<double>(const double*, const double*, const double*, const double*,
                                                double*, int, int, int, tridi_stream_t);

}  // namespace tridi

extern "C" {

tridi_status tridi_pcr_thomas_f32(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                                  int m, int gaussian, tridi_stream_t s) {
  return tridi::pcr_thomas_device<float>(a, b, c, d, x, n, m, gaussian, s);
}
tridi_status tridi_pcr_thomas_f64(const double* a, const double* b, const double* c, const double* d, double* x,
                                  int n, int m, int gaussian, tridi_stream_t s) {
  return tridi::pcr_thomas_device<double>(a, b, c, d, x, n, m, gaussian, s);
}

}  // extern "C"

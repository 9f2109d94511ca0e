// Mixed-precision iterative refinement: FP32 solves, FP64 residual and FP64
// accumulation of the corrections.  No counterpart in the reference (its
// solvers are FP32 or FP64 throughout, common.h:8-12); the oracle is the gold
// Thomas solver run in FP64 (tridiagonal_gold.h:26-44).
//
//   e0 = solve32(T, d)
//   sweep k = 0, 1, ...:
//     x_{k+1} = x_k + e_k                 (FP64; x_0 = 0)
//     r = d - T x_{k+1}                   (FP64; stored as FP32 for the next solve)
//     rel_s = ||r_s|| / ||d_s|| per system; stop when max_s rel_s <= tol
//     e_{k+1} = solve32(T, r)             (the same FP32 kernels as a plain solve)
// The update and the residual are one kernel; x is ping-ponged between two
// 8-byte-per-row buffers so neighbours are read before they are rewritten.
// Only those two steps run in extended precision: native FP64, or (the
// default, TRIDI_TUNE_RESIDUAL) double-float, x held as (hi, lo) FP32 pairs.
// In double-float x_1 = e_0 stays in FP32 and the second sweep writes
// x_2 = e_0 + e_1 straight to FP64 (one correction: no pair buffer, no
// assembly pass); further sweeps run on pairs, assembled into FP64 at the end.
#include <algorithm>
#include <cmath>

#include "dfloat.cuh"
#include "runtime.h"
#include "tridi_device.cuh"

namespace tridi {

template <class T>
tridi_status hybrid_solve_device(const T*, const T*, const T*, const T*, T*, int, int, int, tridi_stream_t);
template <class T>
tridi_status partition_solve_device(const T*, const T*, const T*, const T*, T*, int, int, tridi_stream_t);
template <class T>
tridi_status large_solve_device(const T*, const T*, const T*, const T*, T*, long, long, int, void*, size_t,
                                tridi_stream_t);

struct RefineParams {
  const float *a, *b, *c, *d;
  const float* e;     // FP32 correction
  const double* xin;  // x_k (ignored when first)
  double* xout;       // x_{k+1} (double-float mode: (hi, lo) FP32 pairs in the same 8 bytes)
  const float* x1f;   // double-float mode 1: x_1 = e_0 in FP32
  int mode;           // double-float mode: 0 first sweep (x_1 = e, not written), 1 second sweep
                      // (x_2 = x1f + e, written as FP64), 2 later sweeps (pairs in, pairs out)
  float* r;           // FP32 copy of the residual
  double* rr;         // per-system sum of r^2 (accumulated)
  double* dd;         // per-system sum of d^2 (accumulated on the first sweep)
  long n, m;
  int layout;
  int first;
  int rows_per_block;  // contiguous: elements per block per system chunk; interleaved: rows per block
};

// x_{k+1} at (i, s) without writing it: x_k + e (or e on the first sweep),
// as a double (FP64 mode) or a double-float pair (double-float mode).
template <bool DF>
struct XNext;
template <>
struct XNext<false> {
  using V = double;
  static constexpr int kMinBlocks = 3;  // blocks an SM of the interleaved residual kernel (80 registers)
  static constexpr int kBatch = 2;      // rows a warp loads ahead there
  __device__ __forceinline__ static V get(const RefineParams& p, long k) {
    return p.first ? (double)p.e[k] : p.xin[k] + (double)p.e[k];
  }
  __device__ __forceinline__ static void put(const RefineParams& p, long k, V v) { p.xout[k] = v; }
  __device__ __forceinline__ static V zero() { return 0.0; }
  // d - T x at row i, and d^2; r in FP64, returned rounded to FP32
  __device__ __forceinline__ static float residual(const RefineParams& p, long i, long k, long stride, V xi,
                                                   float* dsq) {
    const double di = (double)p.d[k];
    double r = di - (double)p.b[k] * xi;
    if (i > 0) r -= (double)p.a[k] * get(p, k - stride);
    if (i < p.n - 1) r -= (double)p.c[k] * get(p, k + stride);
    *dsq = p.d[k] * p.d[k];
    return (float)r;
  }
  // the same from values already loaded (xm / xp: x of the rows above / below)
  __device__ __forceinline__ static float residual_v(long i, long n, float a, float b, float c, float d, V xm, V xi,
                                                     V xp, float* dsq) {
    double r = (double)d - (double)b * xi;
    if (i > 0) r -= (double)a * xm;
    if (i < n - 1) r -= (double)c * xp;
    *dsq = d * d;
    return (float)r;
  }
};
// Double-float x; MODE (p.mode, a compile-time choice of the launch): 0
// x = e, not written; 1 x = x1f + e, written in FP64; 2 pairs in, pairs out.
template <int MODE>
struct XDF {
  using V = float2;
  // blocks an SM and rows a warp loads ahead in the interleaved residual
  // kernel, no form spilling: the first sweep's 2 rows at 64 registers, the
  // second sweep's (which also assembles x in FP64) 1 row at 56 (2 rows at 64
  // spilled, at 80 registers and 3 blocks it ran 5 % slower), later sweeps 2
  // rows at 80
  static constexpr int kMinBlocks = MODE == 2 ? 3 : 4;
  static constexpr int kBatch = MODE == 1 ? 1 : 2;
  __device__ __forceinline__ static V get(const RefineParams& p, long k) {
    if constexpr (MODE == 0) return make_float2(p.e[k], 0.f);
    else if constexpr (MODE == 1) return df_add(make_float2(p.x1f[k], 0.f), p.e[k]);
    else return df_add(reinterpret_cast<const float2*>(p.xin)[k], p.e[k]);
  }
  __device__ __forceinline__ static void put(const RefineParams& p, long k, V v) {
    if constexpr (MODE == 1)
      p.xout[k] = df_to_double(v.x, v.y);
    else if constexpr (MODE == 2)
      reinterpret_cast<float2*>(p.xout)[k] = v;
  }
  __device__ __forceinline__ static V zero() { return make_float2(0.f, 0.f); }
  __device__ __forceinline__ static float residual(const RefineParams& p, long i, long k, long stride, V xi,
                                                   float* dsq) {
    const V xm = i > 0 ? get(p, k - stride) : zero();
    const V xp = i < p.n - 1 ? get(p, k + stride) : zero();
    *dsq = p.d[k] * p.d[k];
    return df_residual(i > 0 ? p.a[k] : 0.f, p.b[k], i < p.n - 1 ? p.c[k] : 0.f, p.d[k], xm, xi, xp);
  }
  // the same from values already loaded (xm / xp zero beyond the system's ends)
  __device__ __forceinline__ static float residual_v(long i, long n, float a, float b, float c, float d, V xm, V xi,
                                                     V xp, float* dsq) {
    *dsq = d * d;
    return df_residual(i > 0 ? a : 0.f, b, i < n - 1 ? c : 0.f, d, xm, xi, xp);
  }
};

// x = e exactly in FP64 (refinement that stops after its first sweep).
__global__ void __launch_bounds__(256) refine_f32_to_fp64_kernel(const float* src, double* dst, long count) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x)
    dst[k] = f2d_exact(src[k]);
}

// FP64 x split into normalised double-float pairs (a third sweep after the
// second wrote x in FP64; rare): hi = x rounded to FP32, lo = the rest.
__global__ void __launch_bounds__(256) refine_fp64_to_df_kernel(const double* src, float2* dst, long count) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
    const double v = src[k];
    const float hi = __double2float_rn(v);
    dst[k] = make_float2(hi, __double2float_rn(v - (double)hi));
  }
}

// The final double-float x assembled into FP64 (in place when src == dst:
// each element is read before it is written, by the same thread).
__global__ void __launch_bounds__(256) refine_df_to_fp64_kernel(const float2* src, double* dst, long count) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
    const float2 v = src[k];
    dst[k] = df_to_double(v.x, v.y);
  }
}

// Contiguous layout: block (system s, chunk q) covers rows [q*R, q*R + R).
// Per-thread norm partial sums in FP32 (a few rows each), the block's sums
// in FP64.
template <class X>
__global__ void __launch_bounds__(256) refine_contig_kernel(RefineParams p) {
  const long chunks = (p.n + p.rows_per_block - 1) / p.rows_per_block;
  const long s = blockIdx.x / chunks, q = blockIdx.x % chunks;
  float rsf = 0.f, dsf = 0.f;
  const long i0 = q * p.rows_per_block;
  const long i1 = i0 + p.rows_per_block < p.n ? i0 + p.rows_per_block : p.n;
  for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const long k = s * p.n + i;
    const typename X::V xi = X::get(p, k);
    float dsq;
    const float r = X::residual(p, i, k, 1, xi, &dsq);
    X::put(p, k, xi);
    p.r[k] = r;
    rsf = fmaf(r, r, rsf);
    dsf += dsq;
  }
  double rs = rsf, ds = dsf;
  __shared__ double red[2][8];
  for (int o = 16; o > 0; o >>= 1) {
    rs += __shfl_down_sync(kFull, rs, o);
    ds += __shfl_down_sync(kFull, ds, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = rs;
    red[1][threadIdx.x >> 5] = ds;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0, a1 = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a0 += red[0][w];
      a1 += red[1][w];
    }
    atomicAdd(&p.rr[s], a0);
    if (p.first) atomicAdd(&p.dd[s], a1);
  }
}

// Interleaved layout: block = 32 systems x 8 warps, rows [q*R, q*R + R);
// warp w takes the R/8 contiguous rows from q*R + w*R/8, lane l system
// 32g + l (each row of a warp one 128-byte segment of every array).  x of the
// rows above and below rides along in registers, so each x is formed once;
// rows go in batches of kBatch whose loads are all issued before any of their
// residuals (the stores of r and x alias nothing the loads read, but the
// compiler cannot know that), so a warp keeps kBatch rows of loads in flight.
// Measured on 1024 x 65536, one refinement: double-float 1.76 ms and FP64
// 3.50 ms with the per-form settings below, against 1.91 / 4.09 ms for one row
// at a time with x of every neighbour reloaded (four rows at two blocks an SM:
// 2.07 / 3.79 ms).
template <class X>
__global__ void __launch_bounds__(256, X::kMinBlocks) refine_inter_kernel(RefineParams p) {
  constexpr int kBatch = X::kBatch;
  using V = typename X::V;
  const long groups = (p.m + 31) / 32;
  const long g = blockIdx.x % groups, q = blockIdx.x / groups;
  const long s = g * 32 + (threadIdx.x & 31);
  const int lr = threadIdx.x >> 5;
  const long m = p.m;
  float rsf = 0.f, dsf = 0.f;
  const long wrows = p.rows_per_block / 8;
  const long i0 = q * p.rows_per_block + lr * wrows;
  const long i1 = i0 + wrows < p.n ? i0 + wrows : p.n;
  if (s < m && i0 < i1) {
    V xm = i0 > 0 ? X::get(p, (i0 - 1) * m + s) : X::zero();
    V xi = X::get(p, i0 * m + s);
    for (long ib = i0; ib < i1; ib += kBatch) {
      const long kb = ib * m + s;  // element of row ib; row ib + u is kb + u * m
      float a[kBatch], b[kBatch], c[kBatch], d[kBatch];
      V xn[kBatch];  // x of row ib + u + 1
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (ib + u < i1) {
          const long k = kb + u * m;
          a[u] = __ldg(p.a + k); b[u] = __ldg(p.b + k); c[u] = __ldg(p.c + k); d[u] = __ldg(p.d + k);
          xn[u] = ib + u < p.n - 1 ? X::get(p, k + m) : X::zero();
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (ib + u < i1) {
          const long k = kb + u * m;
          float dsq;
          const float r = X::residual_v(ib + u, p.n, a[u], b[u], c[u], d[u], xm, xi, xn[u], &dsq);
          X::put(p, k, xi);
          p.r[k] = r;
          rsf = fmaf(r, r, rsf);
          dsf += dsq;
          xm = xi;
          xi = xn[u];
        }
      }
    }
  }
  const double rs = rsf, ds = dsf;
  __shared__ double red[2][8][32];
  red[0][lr][threadIdx.x & 31] = rs;
  red[1][lr][threadIdx.x & 31] = ds;
  __syncthreads();
  if (lr == 0 && s < m) {
    double a0 = 0, a1 = 0;
    for (int w = 0; w < 8; ++w) {
      a0 += red[0][w][threadIdx.x];
      a1 += red[1][w][threadIdx.x];
    }
    atomicAdd(&p.rr[s], a0);
    if (p.first) atomicAdd(&p.dd[s], a1);
  }
}

// max over systems of sqrt(rr/dd) into out[0].
__global__ void refine_maxrel_kernel(const double* rr, const double* dd, long m, double* out) {
  double v = 0.0;
  for (long s = threadIdx.x; s < m; s += blockDim.x) {
    const double den = dd[s] > 0 ? dd[s] : 1.0;
    const double q = sqrt(rr[s] / den);
    v = q > v || q != q ? q : v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_down_sync(kFull, v, o);
    v = w > v || w != w ? w : v;
  }
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double w = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) w = red[i] > w || red[i] != red[i] ? red[i] : w;
    out[0] = w;
  }
}

namespace {

long align64(long v) { return (v + 63) & ~63L; }

// Workspace layout (bytes): e (4 nm), e2 (4 nm), r (4 nm), xalt (8 nm), rr (8 m),
// dd (8 m), scalar (8), then the large solver's workspace if needed.
struct RefineWs {
  float* e;
  float* e2;  // double-float mode: the first correction (e holds x_1 = e_0 meanwhile)
  float* r;
  double* xalt;
  double* rr;
  double* dd;
  double* scalar;
  void* inner;
  size_t inner_bytes;
};

bool needs_large(long n, long m, int layout) {
  (void)m;
  return layout == TRIDI_LAYOUT_INTERLEAVED || n > 8704;
}

size_t inner_bytes(long n, long m, int layout) {
  return needs_large(n, m, layout) ? tridi_large_workspace_bytes(n, m, 4) : 0;
}

size_t refine_ws_bytes(long n, long m, int layout) {
  const long nm = align64(n * m);
  return (size_t)nm * (4 + 4 + 4 + 8) + (size_t)align64(m) * 16 + 256 + inner_bytes(n, m, layout) + 1024;
}

RefineWs carve(void* ws, long n, long m, int layout) {
  char* w = static_cast<char*>(ws);
  const long nm = align64(n * m);
  RefineWs r;
  r.e = reinterpret_cast<float*>(w); w += nm * 4;
  r.e2 = reinterpret_cast<float*>(w); w += nm * 4;
  r.r = reinterpret_cast<float*>(w); w += nm * 4;
  r.xalt = reinterpret_cast<double*>(w); w += nm * 8;
  r.rr = reinterpret_cast<double*>(w); w += align64(m) * 8;
  r.dd = reinterpret_cast<double*>(w); w += align64(m) * 8;
  r.scalar = reinterpret_cast<double*>(w); w += 256;
  r.inner = w;
  r.inner_bytes = inner_bytes(n, m, layout);
  return r;
}

int default_rest(int n) {
  const int t = tunable(TRIDI_TUNE_CRPCR_REST);
  const int a = tuned(TRIDI_AUTOTUNE_CRPCR_REST, ilog2(n));
  int rest = t > 0 ? t : (a > 0 ? a : 4);
  while (rest > n / 2 && rest > 2) rest /= 2;
  return rest;
}

// The FP32 solve used for the first solution and every correction.
tridi_status solve32(const float* a, const float* b, const float* c, const float* rhs, float* out, long n, long m,
                     int layout, const RefineWs& w, tridi_stream_t s) {
  if (needs_large(n, m, layout)) return large_solve_device<float>(a, b, c, rhs, out, n, m, layout, w.inner,
                                                                   w.inner_bytes, s);
  if (is_pow2(n) && n >= 4 && n <= 4096)
    return hybrid_solve_device<float>(a, b, c, rhs, out, (int)n, (int)m, (int)n / default_rest((int)n), s);
  return partition_solve_device<float>(a, b, c, rhs, out, (int)n, (int)m, s);
}

}  // namespace

tridi_status refine_device(const float* a, const float* b, const float* c, const float* d, double* x, long n, long m,
                           int layout, double tol, int max_sweeps, void* ws, size_t ws_bytes, tridi_stream_t stream,
                           int* sweeps_out, double* res_out) {
  if (!a || !b || !c || !d || !x || n <= 0 || m <= 0 || max_sweeps < 0 || (layout != 0 && layout != 1))
    return TRIDI_ERROR_INVALID_VALUE;
  if (!ws || ws_bytes < refine_ws_bytes(n, m, layout)) return TRIDI_ERROR_WORKSPACE_TOO_SMALL;
  if (!current_device()) return TRIDI_ERROR_CUDA;
  const RefineWs w = carve(ws, n, m, layout);
  cudaStream_t st = as_stream(stream);
  cudaError_t e;
  const int res = tunable(TRIDI_TUNE_RESIDUAL);
  if (res != 0 && res != TRIDI_RESIDUAL_DF && res != TRIDI_RESIDUAL_FP64) return TRIDI_ERROR_INVALID_VALUE;
  const bool df = res != TRIDI_RESIDUAL_FP64;
  tridi_status ts = solve32(a, b, c, d, w.e, n, m, layout, w, stream);
  if (ts != TRIDI_SUCCESS) return ts;
  if ((e = cudaMemsetAsync(w.dd, 0, sizeof(double) * m, st)) != cudaSuccess) return cuda_status(e);

  RefineParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.e = w.e; p.r = w.r; p.rr = w.rr; p.dd = w.dd;
  p.n = n; p.m = m; p.layout = layout;
  double rel = 0.0;
  // One update + residual pass over the batch with the current p, then the
  // maximum relative residual read back into rel.
  const auto pass = [&]() -> cudaError_t {
    cudaError_t ce;
    if ((ce = cudaMemsetAsync(w.rr, 0, sizeof(double) * m, st)) != cudaSuccess) return ce;
    unsigned blocks;
    if (layout == 0) {
      p.rows_per_block = n < 2048 ? (int)n : 2048;
      const long chunks = (n + p.rows_per_block - 1) / p.rows_per_block;
      blocks = (unsigned)(m * chunks);
      if (!df)
        refine_contig_kernel<XNext<false>><<<blocks, 256, 0, st>>>(p);
      else if (p.mode == 0)
        refine_contig_kernel<XDF<0>><<<blocks, 256, 0, st>>>(p);
      else if (p.mode == 1)
        refine_contig_kernel<XDF<1>><<<blocks, 256, 0, st>>>(p);
      else
        refine_contig_kernel<XDF<2>><<<blocks, 256, 0, st>>>(p);
    } else {
      p.rows_per_block = 256;
      const long groups = (m + 31) / 32, chunks = (n + 255) / 256;
      blocks = (unsigned)(groups * chunks);
      if (!df)
        refine_inter_kernel<XNext<false>><<<blocks, 256, 0, st>>>(p);
      else if (p.mode == 0)
        refine_inter_kernel<XDF<0>><<<blocks, 256, 0, st>>>(p);
      else if (p.mode == 1)
        refine_inter_kernel<XDF<1>><<<blocks, 256, 0, st>>>(p);
      else
        refine_inter_kernel<XDF<2>><<<blocks, 256, 0, st>>>(p);
    }
    refine_maxrel_kernel<<<1, 1024, 0, st>>>(w.rr, w.dd, m, w.scalar);
    if ((ce = cudaGetLastError()) != cudaSuccess) return ce;
    if ((ce = cudaMemcpyAsync(&rel, w.scalar, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return ce;
    return cudaStreamSynchronize(st);
  };
  const auto done = [&](int sw) { return rel <= tol || sw >= max_sweeps || !(rel == rel); };
  const long count = n * m;
  const unsigned eblocks = (unsigned)std::min<long>((count + 255) / 256, 65535L * 8);
  int sweep = 0;
  if (df) {
    // Double-float.  Sweep 0: x_1 = e_0 stays in w.e (FP32, exact), only r_1
    // is written.  Sweep 1: x_2 = e_0 + e_1 (an exact pair) goes to x in FP64
    // directly, so one correction (the usual case) needs no pair buffer and
    // no assembly pass.  Later sweeps (rare) split x into pairs again and run
    // on pairs, assembled into FP64 at the end.
    p.first = 1;
    p.mode = 0;
    if ((e = pass()) != cudaSuccess) return cuda_status(e);
    if (done(0)) {
      refine_f32_to_fp64_kernel<<<eblocks, 256, 0, st>>>(w.e, x, count);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    } else {
      sweep = 1;
      if ((ts = solve32(a, b, c, w.r, w.e2, n, m, layout, w, stream)) != TRIDI_SUCCESS) return ts;
      p.first = 0;
      p.mode = 1;
      p.x1f = w.e;
      p.e = w.e2;
      p.xout = x;
      if ((e = pass()) != cudaSuccess) return cuda_status(e);
      if (!done(1)) {
        refine_fp64_to_df_kernel<<<eblocks, 256, 0, st>>>(x, reinterpret_cast<float2*>(w.xalt), count);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
        // x_k alternates between the workspace copy and x (neighbours are
        // read before they are rewritten)
        double* bufs[2] = {x, w.xalt};
        int cur = 1;
        p.mode = 2;
        p.e = w.e;
        for (sweep = 2;; ++sweep) {
          if ((ts = solve32(a, b, c, w.r, w.e, n, m, layout, w, stream)) != TRIDI_SUCCESS) return ts;
          p.xin = bufs[cur];
          p.xout = bufs[cur ^ 1];
          if ((e = pass()) != cudaSuccess) return cuda_status(e);
          cur ^= 1;
          if (done(sweep)) break;
        }
        // x_k as double-float pairs in bufs[cur] -> FP64 in x
        refine_df_to_fp64_kernel<<<eblocks, 256, 0, st>>>(reinterpret_cast<const float2*>(bufs[cur]), x, count);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
      }
    }
  } else {
    // Native FP64: x_k alternates between the workspace copy and x; the first
    // update writes the workspace, so one correction ends in x.
    double* bufs[2] = {x, w.xalt};
    int cur = 0;  // x_k lives in bufs[cur]
    for (;; ++sweep) {
      p.first = sweep == 0;
      p.xin = bufs[cur];
      p.xout = bufs[cur ^ 1];
      if ((e = pass()) != cudaSuccess) return cuda_status(e);
      cur = (p.xout == x) ? 0 : 1;
      if (done(sweep)) break;
      if ((ts = solve32(a, b, c, w.r, w.e, n, m, layout, w, stream)) != TRIDI_SUCCESS) return ts;
    }
    if (cur != 0 &&
        (e = cudaMemcpyAsync(x, bufs[cur], sizeof(double) * n * m, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
      return cuda_status(e);
  }
  if (sweeps_out) *sweeps_out = sweep;
  if (res_out) *res_out = rel;
  return rel <= tol ? TRIDI_SUCCESS : TRIDI_ERROR_NOT_CONVERGED;
}

}  // namespace tridi

extern "C" {

size_t tridi_refine_workspace_bytes(long n, long num_systems, int layout) {
  return tridi::refine_ws_bytes(n, num_systems, layout);
}

tridi_status tridi_refine_f32(const float* a, const float* b, const float* c, const float* d, double* x, long n,
                              long m, int layout, double tol, int max_sweeps, void* ws, size_t ws_bytes,
                              tridi_stream_t s, int* sweeps, double* rel_residual) {
  return tridi::refine_device(a, b, c, d, x, n, m, layout, tol, max_sweeps, ws, ws_bytes, s, sweeps, rel_residual);
}

}  // extern "C"

// Large systems (any n, contiguous or interleaved layout): the partition
// method across the whole GPU, in three steps on one stream.
//
//   1. large_reduce: one thread per chunk of L rows of one system.  The chunk
//      is eliminated in registers (partition.cuh) and its interface -- first
//      and last interior row coefficients and the separator row, 10 values --
//      is written out.  In the interleaved layout (element i of system s at
//      i*m + s) a warp covers 32 consecutive systems at the same rows, so
//      every row load is one 128-byte line.
//   2. large_assemble: separator row j of system s from chunk j's interface
//      and chunk j+1's first interior row, in the layout of the data.  The
//      P = ceil(n/L) separators per system form a batch of the same kind,
//      solved by the uniform partition solver (contiguous, P <= 8704 in FP32,
//      4608 in FP64) or by
//      this scheme again (interleaved, or larger P), down to a one-thread-
//      per-system Thomas kernel for interleaved batches of <= 32 rows.
//   3. large_back: each chunk is read and eliminated again and its rows
//      recovered from the two separators around it.
// For the interleaved FP32 layout with m a multiple of 32, steps 1 and 3 run
// as TMA-tiled persistent kernels (large_tma.cu) on the same chunks.
// Memory traffic per unknown: inputs read twice (2 x 16 B FP32), x written
// once (4 B), plus ~20/L B of interface data.  No reference kernel
// corresponds; the reference's large-system path is pcrGauss's global-memory
// PCR steps (pcrGauss_kernel.cu:272-386).  Oracle: the gold Thomas solver.
#include "partition.cuh"
#include "runtime.h"

namespace tridi {

template <class T>
tridi_status partition_solve_device(const T* a, const T* b, const T* c, const T* d, T* x, int n, int m,
                                    tridi_stream_t stream);
bool large_tma_ok(const float* a, const float* b, const float* c, const float* d, long n, long m);
tridi_status large_tma_pass(bool back, const float* a, const float* b, const float* c, const float* d, long n,
                            long m, long P, long PMp, float* red, float* bnd, const float* sol, float* x,
                            cudaStream_t st);

struct LargeParams {
  const void* a;
  const void* b;
  const void* c;
  const void* d;
  void* x;
  long n, m;
  long P;       // chunks per system
  int layout;   // 0 contiguous, 1 interleaved
  void* iface;  // 10 arrays of P*m interface values (stride PMp), same layout as the data
  void* red;    // 4 arrays (stride PMp): the separator system, same layout as the data
  long PMp;     // P*m rounded up to 64 elements: keeps each array 256-byte aligned
  void* sol;    // the separator solution (aliases iface), same layout
};

// Thread -> (system, chunk).  Interleaved: systems fastest; contiguous:
// chunks fastest.  Either way consecutive threads touch consecutive
// addresses of the interface and separator arrays, whose layout follows the
// data's: index j*m + s (interleaved) or s*P + j (contiguous).
__device__ __forceinline__ void large_coords(const LargeParams& p, long gid, long* s, long* j) {
  if (p.layout == 1) {
    *s = gid % p.m;
    *j = gid / p.m;
  } else {
    *j = gid % p.P;
    *s = gid / p.P;
  }
}
__device__ __forceinline__ long sep_index(const LargeParams& p, long s, long j) {
  return p.layout == 1 ? j * p.m + s : s * p.P + j;
}

template <class T, int L>
__global__ void __launch_bounds__(256) large_reduce_kernel(LargeParams p) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= p.P * p.m) return;
  long s, j;
  large_coords(p, gid, &s, &j);
  const long r0 = j * L;
  const int k = (int)((p.n - r0) < L ? (p.n - r0) : L);
  const long rs = p.layout == 1 ? p.m : 1;
  const long base = p.layout == 1 ? r0 * p.m + s : s * p.n + r0;
  Chunk<T, L> ch;
  chunk_eliminate<T, L, true>(ch, k, j == 0, j == p.P - 1, static_cast<const T*>(p.a) + base,
                        static_cast<const T*>(p.b) + base, static_cast<const T*>(p.c) + base,
                        static_cast<const T*>(p.d) + base, rs);
  T* f = static_cast<T*>(p.iface);
  const long S = p.PMp, o = sep_index(p, s, j);
  f[0 * S + o] = ch.fD; f[1 * S + o] = ch.fC; f[2 * S + o] = ch.fA;
  f[3 * S + o] = ch.lD; f[4 * S + o] = ch.lC; f[5 * S + o] = ch.lA;
  f[6 * S + o] = ch.sep.a; f[7 * S + o] = ch.sep.b; f[8 * S + o] = ch.sep.c; f[9 * S + o] = ch.sep.d;
}

template <class T>
__global__ void __launch_bounds__(256) large_assemble_kernel(LargeParams p) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= p.P * p.m) return;
  long s, j;
  large_coords(p, gid, &s, &j);
  const T* f = static_cast<const T*>(p.iface);
  const long S = p.PMp, o = sep_index(p, s, j);
  T nD = T(0), nC = T(0), nA = T(0);
  if (j + 1 < p.P) {
    const long o1 = sep_index(p, s, j + 1);
    nD = f[0 * S + o1]; nC = f[1 * S + o1]; nA = f[2 * S + o1];
  }
  const T lD = f[3 * S + o], lC = f[4 * S + o], lA = f[5 * S + o];
  const T sa = f[6 * S + o], sb = f[7 * S + o], sc = f[8 * S + o], sd = f[9 * S + o];
  T* r = static_cast<T*>(p.red);
  r[0 * S + o] = -sa * lA;
  r[1 * S + o] = sb - sa * lC - sc * nA;
  r[2 * S + o] = -sc * nC;
  r[3 * S + o] = sd - sa * lD - sc * nD;
}

template <class T, int L>
__global__ void __launch_bounds__(256) large_back_kernel(LargeParams p) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= p.P * p.m) return;
  long s, j;
  large_coords(p, gid, &s, &j);
  const long r0 = j * L;
  const int k = (int)((p.n - r0) < L ? (p.n - r0) : L);
  const long rs = p.layout == 1 ? p.m : 1;
  const long base = p.layout == 1 ? r0 * p.m + s : s * p.n + r0;
  Chunk<T, L> ch;
  chunk_eliminate<T, L, true>(ch, k, j == 0, j == p.P - 1, static_cast<const T*>(p.a) + base,
                        static_cast<const T*>(p.b) + base, static_cast<const T*>(p.c) + base,
                        static_cast<const T*>(p.d) + base, rs);
  const T* sol = static_cast<const T*>(p.sol);
  const T sj = sol[sep_index(p, s, j)];
  const T sl = j > 0 ? sol[sep_index(p, s, j - 1)] : T(0);
  T x[L];
  chunk_back<T, L>(ch, k, sj, sl, x);
  T* gx = static_cast<T*>(p.x) + base;
#pragma unroll
  for (int i = 0; i < L; ++i)
    if (i < k) gx[i * rs] = x[i];
}

// Base case for interleaved systems: one thread per system runs the gold
// Thomas recurrence (tridiagonal_gold.h:26-44, a[0] and c[n-1] ignored),
// keeping c' and d' in a scratch array; a warp reads 32 consecutive systems,
// so every row access is coalesced.
template <class T>
__global__ void __launch_bounds__(256) thomas_interleaved_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                                 const T* __restrict__ c, const T* __restrict__ d,
                                                                 T* __restrict__ x, long n, long m,
                                                                 T* __restrict__ cp, T* __restrict__ dp) {
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= m) return;
  T cprev = T(0), dprev = T(0);
  for (long i = 0; i < n; ++i) {
    const long k = i * m + s;
    const T ai = i == 0 ? T(0) : a[k];
    const T ci = i == n - 1 ? T(0) : c[k];
    const T inv = tdiv(T(1), b[k] - ai * cprev);
    cprev = ci * inv;
    dprev = (d[k] - ai * dprev) * inv;
    cp[k] = cprev;
    dp[k] = dprev;
  }
  T xn = dprev;
  x[(n - 1) * m + s] = xn;
  for (long i = n - 2; i >= 0; --i) {
    const long k = i * m + s;
    xn = dp[k] - cp[k] * xn;
    x[k] = xn;
  }
}

namespace {
constexpr int kChunk = 16;
// Interleaved base case: one thread per system, a serial chain over n rows
// with only m threads in flight, so it is kept short (the recursion goes one
// level further rather than run 256-row chains on 1024 threads).
constexpr long kThomasMax = 32;

long round64(long v) { return (v + 63) & ~63L; }

// Workspace of one level plus the levels below it.
template <class T>
size_t large_ws_bytes(long n, long m, int layout) {
  if (layout == 1 && n <= kThomasMax) return (size_t)2 * round64(n * m) * sizeof(T) + 256;
  const long P = (n + kChunk - 1) / kChunk;
  size_t own = (size_t)14 * round64(P * m) * sizeof(T) + 256;
  if (layout == 1 || P > partition_max_rows<T>()) own += large_ws_bytes<T>(P, m, layout);
  return own;
}
}  // namespace

template <class T>
size_t large_workspace_bytes(long n, long m, int layout) {
  return large_ws_bytes<T>(n, m, layout);
}
template size_t large_workspace_bytes<float>(long, long, int);
template size_t large_workspace_bytes<double>(long, long, int);

template <class T>
tridi_status large_solve_device(const T* a, const T* b, const T* c, const T* d, T* x, long n, long m, int layout,
                                void* ws, size_t ws_bytes, tridi_stream_t stream) {
  if (!a || !b || !c || !d || !x || m <= 0 || n <= 0 || (layout != 0 && layout != 1))
    return TRIDI_ERROR_INVALID_VALUE;
  if (n * m > (1L << 34)) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  if (!ws || ws_bytes < large_ws_bytes<T>(n, m, layout)) return TRIDI_ERROR_WORKSPACE_TOO_SMALL;
  if (!current_device()) return TRIDI_ERROR_CUDA;
  cudaStream_t st = as_stream(stream);
  char* w = static_cast<char*>(ws);
  if (layout == 1 && n <= kThomasMax) {
    T* cp = reinterpret_cast<T*>(w);
    T* dp = cp + round64(n * m);
    thomas_interleaved_kernel<T><<<(unsigned)((m + 255) / 256), 256, 0, st>>>(a, b, c, d, x, n, m, cp, dp);
    return cuda_status(cudaGetLastError());
  }
  LargeParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.layout = layout;
  p.P = (n + kChunk - 1) / kChunk;
  const long PM = p.P * m;
  p.PMp = round64(PM);
  p.iface = w;
  p.red = w + (size_t)10 * p.PMp * sizeof(T);
  p.sol = w;  // the interface is dead once the separator rows are assembled
  void* inner = w + (size_t)14 * p.PMp * sizeof(T) + 256;
  const size_t inner_bytes = ws_bytes - ((size_t)14 * p.PMp * sizeof(T) + 256);
  const unsigned blocks = (unsigned)((PM + 255) / 256);
  // interleaved FP32 with m a multiple of 32: the TMA-tiled passes (large_tma.cu)
  bool tma = false;
  if constexpr (sizeof(T) == 4)
    tma = layout == 1 && tunable(TRIDI_TUNE_LARGE_TMA) != 2 && !g_host_mapped_io && large_tma_ok(a, b, c, d, n, m);
  if (tma) {
    // the separator rows assembled in the pass (the interface area holds the
    // tile-boundary arrays only)
    const tridi_status t = large_tma_pass(false, reinterpret_cast<const float*>(a), reinterpret_cast<const float*>(b),
                                          reinterpret_cast<const float*>(c), reinterpret_cast<const float*>(d), n, m,
                                          p.P, p.PMp, static_cast<float*>(p.red), static_cast<float*>(p.iface),
                                          nullptr, nullptr, st);
    if (t != TRIDI_SUCCESS) return t;
  } else {
    large_reduce_kernel<T, kChunk><<<blocks, 256, 0, st>>>(p);
    large_assemble_kernel<T><<<blocks, 256, 0, st>>>(p);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  const T* r = static_cast<const T*>(p.red);
  tridi_status ts;
  if (layout == 0 && p.P <= partition_max_rows<T>())
    ts = partition_solve_device<T>(r, r + p.PMp, r + 2 * p.PMp, r + 3 * p.PMp, static_cast<T*>(p.sol), (int)p.P,
                                   (int)m, stream);
  else
    ts = large_solve_device<T>(r, r + p.PMp, r + 2 * p.PMp, r + 3 * p.PMp, static_cast<T*>(p.sol), p.P, m, layout,
                               inner, inner_bytes, stream);
  if (ts != TRIDI_SUCCESS) return ts;
  if (tma)
    return large_tma_pass(true, reinterpret_cast<const float*>(a), reinterpret_cast<const float*>(b),
                          reinterpret_cast<const float*>(c), reinterpret_cast<const float*>(d), n, m, p.P, p.PMp,
                          nullptr, nullptr, static_cast<const float*>(p.sol), reinterpret_cast<float*>(x), st);
  large_back_kernel<T, kChunk><<<blocks, 256, 0, st>>>(p);
  return cuda_status(cudaGetLastError());
}

template tridi_status large_solve_device<float>(const float*, const float*, const float*, const float*, float*, long,
                                                long, int, void*, size_t, tridi_stream_t);
template tridi_status large_solve_device<double>(const double*, const double*, const double*, const double*,
                                                 double*, long, long, int, void*, size_t, tridi_stream_t);

}  // namespace tridi

extern "C" {

size_t tridi_large_workspace_bytes(long n, long num_systems, int elem_size) {
  // the larger of the two layouts' needs, so one query serves both
  const size_t c0 = elem_size == 8 ? tridi::large_ws_bytes<double>(n, num_systems, 0)
                                   : tridi::large_ws_bytes<float>(n, num_systems, 0);
  const size_t c1 = elem_size == 8 ? tridi::large_ws_bytes<double>(n, num_systems, 1)
                                   : tridi::large_ws_bytes<float>(n, num_systems, 1);
  return c0 > c1 ? c0 : c1;
}
tridi_status tridi_solve_large_f32(const float* a, const float* b, const float* c, const float* d, float* x, long n,
                                   long m, int layout, void* ws, size_t ws_bytes, tridi_stream_t s) {
  return tridi::large_solve_device<float>(a, b, c, d, x, n, m, layout, ws, ws_bytes, s);
}
tridi_status tridi_solve_large_f64(const double* a, const double* b, const double* c, const double* d, double* x,
                                   long n, long m, int layout, void* ws, size_t ws_bytes, tridi_stream_t s) {
  return tridi::large_solve_device<double>(a, b, c, d, x, n, m, layout, ws, ws_bytes, s);
}

}  // extern "C"

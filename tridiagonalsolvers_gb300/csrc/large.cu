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
//      and chunk j+1's first interior row, written contiguously per system;
//      the P = ceil(n/L) separators of every system are then solved by the
//      uniform partition solver (partition.cu).
//   3. large_back: each chunk is read and eliminated again and its rows
//      recovered from the two separators around it.
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

struct LargeParams {
  const void* a;
  const void* b;
  const void* c;
  const void* d;
  void* x;
  long n, m;
  long P;       // chunks per system
  int L;        // rows per chunk
  int layout;   // 0 contiguous, 1 interleaved
  void* iface;  // 10 arrays of P*m interface values, index j*m + s
  void* red;    // 4 arrays (stride PMp) of separator rows, index s*P + j
  long PMp;     // P*m rounded up to 64 elements: keeps each array 256-byte aligned
  void* sol;    // P*m separator solution, index s*P + j
};

// Thread -> (system, chunk).  Interleaved: systems fastest (coalesced rows).
// Contiguous: chunks fastest (a warp walks one system).
__device__ __forceinline__ void large_coords(const LargeParams& p, long gid, long* s, long* j) {
  if (p.layout == 1) {
    *s = gid % p.m;
    *j = gid / p.m;
  } else {
    *j = gid % p.P;
    *s = gid / p.P;
  }
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
  chunk_eliminate<T, L>(ch, k, j == 0, j == p.P - 1, static_cast<const T*>(p.a) + base,
                        static_cast<const T*>(p.b) + base, static_cast<const T*>(p.c) + base,
                        static_cast<const T*>(p.d) + base, rs);
  T* f = static_cast<T*>(p.iface);
  const long PM = p.P * p.m, o = j * p.m + s;
  f[0 * PM + o] = ch.fD; f[1 * PM + o] = ch.fC; f[2 * PM + o] = ch.fA;
  f[3 * PM + o] = ch.lD; f[4 * PM + o] = ch.lC; f[5 * PM + o] = ch.lA;
  f[6 * PM + o] = ch.sep.a; f[7 * PM + o] = ch.sep.b; f[8 * PM + o] = ch.sep.c; f[9 * PM + o] = ch.sep.d;
}

template <class T>
__global__ void __launch_bounds__(256) large_assemble_kernel(LargeParams p) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= p.P * p.m) return;
  const long s = gid % p.m, j = gid / p.m;  // coalesced interface reads
  const T* f = static_cast<const T*>(p.iface);
  const long PM = p.P * p.m, o = j * p.m + s;
  T nD = T(0), nC = T(0), nA = T(0);
  if (j + 1 < p.P) {
    nD = f[0 * PM + o + p.m]; nC = f[1 * PM + o + p.m]; nA = f[2 * PM + o + p.m];
  }
  const T lD = f[3 * PM + o], lC = f[4 * PM + o], lA = f[5 * PM + o];
  const T sa = f[6 * PM + o], sb = f[7 * PM + o], sc = f[8 * PM + o], sd = f[9 * PM + o];
  T* r = static_cast<T*>(p.red);
  const long q = s * p.P + j, PMp = p.PMp;
  r[0 * PMp + q] = -sa * lA;
  r[1 * PMp + q] = sb - sa * lC - sc * nA;
  r[2 * PMp + q] = -sc * nC;
  r[3 * PMp + q] = sd - sa * lD - sc * nD;
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
  chunk_eliminate<T, L>(ch, k, j == 0, j == p.P - 1, static_cast<const T*>(p.a) + base,
                        static_cast<const T*>(p.b) + base, static_cast<const T*>(p.c) + base,
                        static_cast<const T*>(p.d) + base, rs);
  const T* sol = static_cast<const T*>(p.sol);
  const T sj = sol[s * p.P + j];
  const T sl = j > 0 ? sol[s * p.P + j - 1] : T(0);
  T x[L];
  chunk_back<T, L>(ch, k, sj, sl, x);
  T* gx = static_cast<T*>(p.x) + base;
#pragma unroll
  for (int i = 0; i < L; ++i)
    if (i < k) gx[i * rs] = x[i];
}

namespace {
constexpr int kChunk = 16;

long round64(long v) { return (v + 63) & ~63L; }

template <class T>
size_t large_ws_bytes(long n, long m) {
  const long P = (n + kChunk - 1) / kChunk;
  return (size_t)(10 * P * m + 4 * round64(P * m)) * sizeof(T) + 1024;
}
}  // namespace

template <class T>
tridi_status large_solve_device(const T* a, const T* b, const T* c, const T* d, T* x, long n, long m, int layout,
                                void* ws, size_t ws_bytes, tridi_stream_t stream) {
  if (!a || !b || !c || !d || !x || m <= 0 || n <= 0 || (layout != 0 && layout != 1))
    return TRIDI_ERROR_INVALID_VALUE;
  const long P = (n + kChunk - 1) / kChunk;
  const int pmax = sizeof(T) == 4 ? 8704 : 4608;
  if (P > pmax || P * m > (1L << 31)) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  if (!ws || ws_bytes < large_ws_bytes<T>(n, m)) return TRIDI_ERROR_WORKSPACE_TOO_SMALL;
  if (!current_device()) return TRIDI_ERROR_CUDA;
  LargeParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.P = P; p.L = kChunk; p.layout = layout;
  const long PM = P * m;
  p.PMp = round64(PM);
  char* w = static_cast<char*>(ws);
  const size_t ifb = ((size_t)10 * PM * sizeof(T) + 255) & ~size_t(255);
  p.iface = w;
  p.red = w + ifb;
  p.sol = w;  // the interface is dead once the separator rows are assembled
  cudaStream_t st = as_stream(stream);
  const unsigned blocks = (unsigned)((PM + 255) / 256);
  large_reduce_kernel<T, kChunk><<<blocks, 256, 0, st>>>(p);
  large_assemble_kernel<T><<<blocks, 256, 0, st>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  const T* r = static_cast<const T*>(p.red);
  tridi_status ts = partition_solve_device<T>(r, r + p.PMp, r + 2 * p.PMp, r + 3 * p.PMp, static_cast<T*>(p.sol),
                                              (int)P, (int)m, stream);
  if (ts != TRIDI_SUCCESS) return ts;
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
  return elem_size == 8 ? tridi::large_ws_bytes<double>(n, num_systems)
                        : tridi::large_ws_bytes<float>(n, num_systems);
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

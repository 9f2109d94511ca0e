// TMA-tiled passes of the large-system solver for the interleaved FP32
// layout (element i of system s at i*m + s, m a multiple of 32).
//
// The two passes of large.cu that read the coefficients -- large_reduce
// (chunk elimination, interface out) and large_back (elimination again, back
// substitution, x out) -- as persistent kernels: one CTA per SM, a producer
// warp that streams tiles of kTileRows rows x 32 systems of a, b, c, d into a
// kStages-deep shared-memory ring with cp.async.bulk.tensor.2d (one tensor
// map per array), and 8 consumer warps.  Warp w of a tile owns rows
// [w*16, w*16 + 16) of it, lane l system s0 + l: exactly the chunks (16 rows
// of one system) of the register kernels, so the interface arrays, the
// separator assembly and the recursion are shared with them.  A lane reads
// its column of the tile (row stride 32 words: lane l always on bank l, no
// conflicts), eliminates it in place, and writes its interface (reduce) or
// its 16 unknowns (back) straight to global memory: consecutive lanes,
// consecutive systems, one 128-byte line per row.
//
// Against the register kernels (one thread per chunk, 64 prefetched values
// and the chunk's eliminated rows in registers, two blocks per SM) the ring
// keeps 128 KB of loads in flight per SM whatever the compute is doing.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "partition.cuh"
#include "runtime.h"

namespace tridi {

namespace {
constexpr int kLtWarps = 8;                  // consumer warps
constexpr int kLtChunk = 16;                 // rows per lane (= the register kernels' chunk)
constexpr int kTileRows = kLtWarps * kLtChunk;  // 128
constexpr int kTileCols = 32;                // systems per tile
constexpr int kStages = 3;
constexpr int kTileFloats = kTileRows * kTileCols;  // per array
constexpr size_t kLtSmem = 128 + (size_t)kStages * 4 * kTileFloats * sizeof(float);  // 192 KB + barriers

struct LtParams {
  long n, m, P, PMp;
  float* red;       // reduce: the separator system, 4 arrays of P*m (stride PMp)
  float* bnd;       // reduce: tile-boundary interface, 10 arrays of row_tiles*m (stride BS)
  long BS;
  const float* sol; // back: separators
  float* x;         // back: solution
  int row_tiles, col_tiles;
  unsigned* status;
};
constexpr int kBndLast = 0;   // bnd arrays 0..6: lD, lC, lA and the separator row of a tile's last chunk
constexpr int kBndFirst = 7;  // bnd arrays 7..9: fD, fC, fA of a tile's first chunk
constexpr size_t kLtExchange = 2 * kLtWarps * 32 * 3 * sizeof(float);  // reduce: fD, fC, fA per lane, two tiles

// Separator row of a chunk (partition.cuh's separator_row_s) from its
// summary and the next chunk's first-row coefficients, into the 4 arrays
// of the separator system at index o.
__device__ __forceinline__ void put_separator(float* red, long S, long o, const Row<float>& sep, float lD, float lC,
                                              float lA, float nD, float nC, float nA) {
  red[0 * S + o] = -sep.a * lA;
  red[1 * S + o] = sep.b - sep.a * lC - sep.c * nA;
  red[2 * S + o] = -sep.c * nC;
  red[3 * S + o] = sep.d - sep.a * lD - sep.c * nD;
}

// Forward elimination of one lane's column (rows 0..k-2 at stride 32 words)
// into registers: the normalised c', a', d' of every interior row.  The
// stage can go back to the producer as soon as this (and the read of the
// separator row) is done.
__device__ __forceinline__ void column_forward(int k, bool first, const float* __restrict__ sa,
                                               const float* __restrict__ sb, const float* __restrict__ sc,
                                               const float* __restrict__ sd, float (&cp)[kLtChunk],
                                               float (&ap)[kLtChunk], float (&dp)[kLtChunk], float& cprev,
                                               float& aprev, float& dprev) {
  cprev = 0.f; aprev = 0.f; dprev = 0.f;
#pragma unroll
  for (int i = 0; i < kLtChunk - 1; ++i) {
    if (i < k - 1) {
      const int o = i * kTileCols;
      const float a = (i == 0 && first) ? 0.f : sa[o];
      const float inv = tdiv(1.f, sb[o] - a * cprev);
      cp[i] = sc[o] * inv;
      ap[i] = (i == 0 ? a : -a * aprev) * inv;
      dp[i] = (sd[o] - a * dprev) * inv;
      cprev = cp[i]; aprev = ap[i]; dprev = dp[i];
    }
  }
}

// The chunk's interface (partition.cuh's Chunk summary) from its eliminated
// rows in registers (last interior row: cl, al, dl).
__device__ __forceinline__ void column_summary(ChunkSummary<float>& cs, int k, const float (&cp)[kLtChunk],
                                               const float (&ap)[kLtChunk], const float (&dp)[kLtChunk], float cl,
                                               float al, float dl) {
  float D = 0.f, C = -1.f, A = 0.f;
#pragma unroll
  for (int i = kLtChunk - 2; i >= 0; --i) {
    if (i <= k - 2) {
      D = dp[i] - cp[i] * D;
      C = -cp[i] * C;
      A = ap[i] - cp[i] * A;
    }
  }
  cs.fD = D; cs.fC = C; cs.fA = A;
  if (k >= 2) {
    cs.lD = dl; cs.lC = cl; cs.lA = al;
  } else {
    cs.lD = 0.f; cs.lC = 0.f; cs.lA = -1.f;
  }
}

template <bool BACK>
__global__ void __launch_bounds__(32 * (kLtWarps + 1), 1)
    large_tile_kernel(LtParams p, const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                      const __grid_constant__ CUtensorMap mc, const __grid_constant__ CUtensorMap md) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + kStages;
  float* ring = reinterpret_cast<float*>(smem + 128);  // stage s, array q at ring + (s*4 + q) * kTileFloats
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ntiles = p.row_tiles * p.col_tiles;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kLtWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (warp == kLtWarps) {  // ---------------- producer ----------------
    if (lane != 0) return;
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int s = k % kStages;
      if (k >= kStages && !mbar_wait(&empty[s], ((k / kStages) - 1) & 1, p.status)) return;
      const int x0 = (t % p.col_tiles) * kTileCols, y0 = (t / p.col_tiles) * kTileRows;
      mbar_arrive_expect_tx(&full[s], 4u * kTileFloats * sizeof(float));
      float* st = ring + (size_t)s * 4 * kTileFloats;
      tma_load_2d(st + 0 * kTileFloats, &ma, x0, y0, &full[s]);
      tma_load_2d(st + 1 * kTileFloats, &mb, x0, y0, &full[s]);
      tma_load_2d(st + 2 * kTileFloats, &mc, x0, y0, &full[s]);
      tma_load_2d(st + 3 * kTileFloats, &md, x0, y0, &full[s]);
    }
    return;
  }

  // ---------------- consumers ----------------
  // (the reduce pass exchanges first-row coefficients between its warps
  // through shared memory, so the consumers agree on every wait's outcome
  // and leave together)
  float* exch = reinterpret_cast<float*>(smem + kLtSmem);
  int k = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
    const int s = k % kStages;
    if (!named_sync_and(1, 32 * kLtWarps, mbar_wait(&full[s], (k / kStages) & 1, p.status))) return;
    const long sys = (long)(t % p.col_tiles) * kTileCols + lane;
    const long r0 = (long)(t / p.col_tiles) * kTileRows + (long)warp * kLtChunk;  // the lane's first row
    const long j = r0 / kLtChunk;                                                 // its chunk
    float* st = ring + (size_t)s * 4 * kTileFloats + warp * kLtChunk * kTileCols + lane;
    float* sa = st;
    float* sb = st + kTileFloats;
    float* sc = st + 2 * kTileFloats;
    float* sd = st + 3 * kTileFloats;
    const long rem = p.n - r0;
    const int kr = rem <= 0 ? 0 : (rem < kLtChunk ? (int)rem : kLtChunk);
    ChunkSummary<float> cs;
    // The eliminated column stays in registers and the stage goes back to
    // the producer right after the elimination, so a stage is held for the
    // elimination only (not for the separator wait and back substitution,
    // nor for the interface exchange).
    float cp[kLtChunk], ap[kLtChunk], dp[kLtChunk];
    float cl = 0.f, al = 0.f, dl = 0.f;
    float sj = 0.f, sl = 0.f;
    if (kr > 0) {
      if constexpr (BACK) {  // the separators' loads overlap the elimination
        const long o = j * p.m + sys;
        sj = p.sol[o];
        sl = j > 0 ? p.sol[o - p.m] : 0.f;
      }
      column_forward(kr, j == 0, sa, sb, sc, sd, cp, ap, dp, cl, al, dl);
      if constexpr (!BACK) {
        const int o = (kr - 1) * kTileCols;
        cs.sep = Row<float>{sa[o], sb[o], sc[o], sd[o]};
        if (kr == 1 && j == 0) cs.sep.a = 0.f;
        if (j == p.P - 1) cs.sep.c = 0.f;
      }
    }
    release_stage(&empty[s]);
    if constexpr (BACK) {
      if (kr > 0) {
        float* gx = p.x + r0 * p.m + sys;
        gx[(long)(kr - 1) * p.m] = sj;
        float xn = sj;
#pragma unroll
        for (int i = kLtChunk - 2; i >= 0; --i) {
          if (i <= kr - 2) {
            xn = dp[i] - cp[i] * xn - ap[i] * sl;
            gx[(long)i * p.m] = xn;
          }
        }
      }
      continue;
    }
    if (kr > 0) column_summary(cs, kr, cp, ap, dp, cl, al, dl);
    if constexpr (!BACK) {
      // separator rows: warp w < 7 takes the next chunk's first row from warp
      // w + 1 of the same tile; a tile's last chunk and its first chunk go to
      // the boundary arrays, assembled by large_tile_boundary_kernel
      float* ex = exch + (k & 1) * (kLtWarps * 32 * 3);
      float* mine = ex + (warp * 32 + lane) * 3;
      mine[0] = kr > 0 ? cs.fD : 0.f;
      mine[1] = kr > 0 ? cs.fC : 0.f;
      mine[2] = kr > 0 ? cs.fA : 0.f;
      consumer_sync(32 * kLtWarps);
      if (kr > 0) {
        const long tr = t / p.col_tiles;
        if (warp + 1 < kLtWarps) {
          const float* nx = ex + ((warp + 1) * 32 + lane) * 3;
          put_separator(p.red, p.PMp, j * p.m + sys, cs.sep, cs.lD, cs.lC, cs.lA, nx[0], nx[1], nx[2]);
        } else {
          float* b = p.bnd + tr * p.m + sys;
          b[(kBndLast + 0) * p.BS] = cs.lD; b[(kBndLast + 1) * p.BS] = cs.lC; b[(kBndLast + 2) * p.BS] = cs.lA;
          b[(kBndLast + 3) * p.BS] = cs.sep.a; b[(kBndLast + 4) * p.BS] = cs.sep.b;
          b[(kBndLast + 5) * p.BS] = cs.sep.c; b[(kBndLast + 6) * p.BS] = cs.sep.d;
        }
        if (warp == 0) {
          float* b = p.bnd + tr * p.m + sys;
          b[(kBndFirst + 0) * p.BS] = cs.fD; b[(kBndFirst + 1) * p.BS] = cs.fC; b[(kBndFirst + 2) * p.BS] = cs.fA;
        }
      }
    }
  }
}

// Separator rows of the tiles' last chunks (chunk 8 tr + 7 of every tile row
// tr), whose next chunk opens the next tile row: one thread per (tr, system).
__global__ void __launch_bounds__(256) large_tile_boundary_kernel(LtParams p) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long)p.row_tiles * p.m) return;
  const long tr = gid / p.m, sys = gid - tr * p.m;
  const long j = tr * kLtWarps + kLtWarps - 1;
  if (j >= p.P) return;  // the system's last chunk lies in an earlier warp of this tile
  const float* b = p.bnd + gid;
  const Row<float> sep{b[(kBndLast + 3) * p.BS], b[(kBndLast + 4) * p.BS], b[(kBndLast + 5) * p.BS],
                       b[(kBndLast + 6) * p.BS]};
  float nD = 0.f, nC = 0.f, nA = 0.f;
  if (j + 1 < p.P) {
    const float* f = b + p.m;  // tile row tr + 1, the same system
    nD = f[(kBndFirst + 0) * p.BS]; nC = f[(kBndFirst + 1) * p.BS]; nA = f[(kBndFirst + 2) * p.BS];
  }
  put_separator(p.red, p.PMp, j * p.m + sys, sep, b[(kBndLast + 0) * p.BS], b[(kBndLast + 1) * p.BS],
                b[(kBndLast + 2) * p.BS], nD, nC, nA);
}

bool make_map(CUtensorMap* map, const float* base, long n, long m) {
  return make_tensor_map_2d(map, base, (uint64_t)m, (uint64_t)n, (uint64_t)m * sizeof(float), kTileCols, kTileRows,
                            false);
}

}  // namespace

// Whether the TMA passes apply: interleaved FP32, m a multiple of 32, 16-byte
// aligned arrays, a chunk count that matches (P = ceil(n / 16)).
bool large_tma_ok(const float* a, const float* b, const float* c, const float* d, long n, long m) {
  return m % kTileCols == 0 && n >= 2 && aligned16(a) && aligned16(b) && aligned16(c) && aligned16(d) &&
         n < (1L << 31) && m < (1L << 31);
}

// Bytes of the boundary arrays of a reduce pass (within the 10 * PMp
// interface floats the register kernels use).
long large_tma_boundary_stride(long n, long m) { return ((((n + kTileRows - 1) / kTileRows) * m) + 63) & ~63L; }

// One TMA pass: back = false -> the separator system (reduce, with the
// assembly of separator rows fused in; bnd: scratch of 10 boundary arrays),
// true -> x (back).
tridi_status large_tma_pass(bool back, const float* a, const float* b, const float* c, const float* d, long n,
                            long m, long P, long PMp, float* red, float* bnd, const float* sol, float* x,
                            cudaStream_t st) {
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  const size_t smem = back ? kLtSmem : kLtSmem + kLtExchange;
  if ((size_t)dev->max_smem_optin < smem) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  CUtensorMap ma, mb, mc, md;
  if (!make_map(&ma, a, n, m) || !make_map(&mb, b, n, m) || !make_map(&mc, c, n, m) || !make_map(&md, d, n, m))
    return TRIDI_ERROR_INVALID_VALUE;
  LtParams p{};
  p.n = n; p.m = m; p.P = P; p.PMp = PMp; p.red = red; p.bnd = bnd; p.sol = sol; p.x = x;
  p.BS = large_tma_boundary_stride(n, m);
  p.row_tiles = (int)((n + kTileRows - 1) / kTileRows);
  p.col_tiles = (int)(m / kTileCols);
  p.status = dev->status;
  const long ntiles = (long)p.row_tiles * p.col_tiles;
  int grid = dev->sm_count;
  if (grid > ntiles) grid = (int)ntiles;
  cudaError_t e;
  if (back) {
    if ((e = cudaFuncSetAttribute(large_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kLtSmem)) != cudaSuccess)
      return cuda_status(e);
    large_tile_kernel<true><<<grid, 32 * (kLtWarps + 1), kLtSmem, st>>>(p, ma, mb, mc, md);
  } else {
    if ((e = cudaFuncSetAttribute(large_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)) != cudaSuccess)
      return cuda_status(e);
    large_tile_kernel<false><<<grid, 32 * (kLtWarps + 1), smem, st>>>(p, ma, mb, mc, md);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    const long cnt = (long)p.row_tiles * m;
    large_tile_boundary_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(p);
  }
  return cuda_status(cudaGetLastError());
}

}  // namespace tridi

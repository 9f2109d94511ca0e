// Ragged batches: systems of different sizes, concatenated (system s owns rows
// [off[s], off[s+1]) of a, b, c, d, x), solved by ONE persistent launch.
// No counterpart in the reference (its launchers take one size per call).
//
// Work queue.  The host plan (tridi_ragged_plan_*) sorts the systems by size
// and cuts them into work items, largest first:
//   SINGLE one system solved by the whole CTA (480 threads)
//   BIG    one system beyond the shared-memory ring (up to 24480 rows), read
//          from global memory by the whole CTA: every thread owns three
//          chunks of up to 17 rows; pass 1 eliminates them and exports their
//          interfaces, the 1440 separators are solved by PCR in shared
//          memory, pass 2 eliminates again (rows now in L2) and substitutes
//          back
//   GROUP  one system solved by a team of 160 threads
//   MULTI  up to 5 systems, one warp each, solved by a team
// Which of 32, 160 or 480 threads a system gets is the autotuner's choice
// for its size bucket (else 32 up to 480 rows, 160 up to 4800, 480 above).
// CTA-wide items (SINGLE, BIG) come first in the list.  One CTA per SM: 480
// consumer threads in 3 teams of 5 warps, and a producer warp.  CTA b takes
// items b, b + grid, b + 2 grid, ... (so every CTA gets the same mix of
// sizes, and no claim has to wait on an atomic); its consumers work through
// the CTA-wide items together, then split into the 3 teams, team t taking
// every third of the remaining items.  Teams overlap one another's loads,
// separator solves and barriers.
//
// Staging.  Shared memory holds a ring of rows (a, b, c, d, and in the
// refined modes the two words of x): the producer places each item's rows
// contiguously at the ring's head (wrapping to row 0 when the tail end is too
// short), copies every system's 16-byte-aligned row range per array with
// cp.async.bulk, and publishes the item in one of kSlots descriptor slots
// through that slot's mbarrier.  Consumers release each slot when done; the
// producer reclaims ring rows oldest first.  So up to kSlots items of any
// size are in flight, and a large item's copy overlaps the solve of the items
// before it.
//
// Arithmetic: the partition solver of partition.cuh, per warp (MULTI), per
// team of 160 threads (GROUP) or per CTA (SINGLE), with the chunk
// elimination done in place in the ring (no register arrays, so no bound on
// rows per thread) and the separators solved by PCR in shuffles (warp), or
// by one warp of the group from shared memory (team and CTA: a 5- or 15-row
// chunk per lane, then PCR in shuffles).
//
// Refined modes (tridi_ragged_refine_f32): every system is refined where it
// sits, without leaving the SM: FP32 solve -> x; then `sweeps` times
// { the original a, c, d re-staged from L2 into the ring, where the FP32
// elimination had overwritten them; FP32 solve of T e = r in the ring, each
// row's residual r = d - T x formed in extended precision as the row is
// eliminated; x += e (extended precision) }; finally, after one more
// re-staging, ||d - T x|| / ||d|| per system (its maximum over the batch goes
// to one device word) and x is written once as FP64.  So HBM sees
// each coefficient once and each unknown once (16 B in, 8 B out per row).
// Extended precision is either native FP64 (RES_FP64) or double-float, an
// unevaluated sum of two FP32 values with a 48-bit significand (RES_DF).
// BIG systems refine the same way with their x and r in a global scratch.
//
// The arrays must hold at least round_up(total_rows, 4) elements and be
// 16-byte aligned (the bulk copies read whole 16-byte groups).
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "dfloat.cuh"
#include "partition.cuh"
#include "runtime.h"

namespace tridi {

constexpr int kRagThreads = 480;       // consumer threads per CTA (15 warps; + 1 producer warp = 16 warps,
                                       // 4 per SM sub-partition, so up to 128 registers per thread)
constexpr int kRagWarps = kRagThreads / 32;
constexpr int kTeams = 3;              // consumer teams (see the file comment)
constexpr int kTeamWarps = kRagWarps / kTeams;      // 5
constexpr int kTeamThreads = 32 * kTeamWarps;       // 160
constexpr int kSlots = 9;              // items in flight (descriptor slots), 3 per team
constexpr int kWarpMaxRows = 480;      // MULTI systems by default: up to 15 rows per lane
constexpr int kGroupMaxRows = 4800;    // GROUP systems by default: up to 30 rows per thread
constexpr int kMaxItemSystems = kTeamWarps;  // 5
static_assert(kTeamWarps & 1, "odd separator rows per lane in warp_solve_rows");
static_assert(kTeams * kTeamWarps == kRagWarps && kSlots % kTeams == 0, "team shape");
constexpr int kBigChunks = 3;                           // chunks per thread for BIG systems
constexpr int kBigSepRows = kBigChunks * kRagThreads;   // chunks (separators) of a BIG system
constexpr int kBigKC = 17;                              // rows per BIG chunk at most
constexpr int kMaxBigRows = kBigKC * kBigSepRows;       // 24480
constexpr int kBigScratchRows = 2 * kBigSepRows;        // ring rows a BIG item borrows as scratch

// MULTI and GROUP items are a team's; SINGLE and BIG take the whole CTA.
enum ItemKind : int { kMulti = 0, kGroup = 1, kSingle = 2, kBig = 3, kEnd = 4 };
// Refined modes: kRefineDF / kRefineFP64 keep x in two extra ring arrays
// (any number of sweeps); the one-correction modes kRefine1DF / kRefine1FP64
// (sweeps == 1) keep the FP32 solution in the b words and the correction in
// the d words, so their ring holds as many rows as the plain one.
enum RagMode : int { kPlain = 0, kRefineDF = 1, kRefineFP64 = 2, kRefine1DF = 3, kRefine1FP64 = 4 };
__host__ __device__ constexpr bool one_correction(int mode) { return mode >= kRefine1DF; }
// DF or FP64: the residual arithmetic of a refined mode
__host__ __device__ constexpr int residual_mode(int mode) {
  return mode == kRefine1DF ? kRefineDF : (mode == kRefine1FP64 ? kRefineFP64 : mode);
}

// Shared-memory map: [head: 2 x kSlots mbarriers, kSlots descriptors]
// [group scratch: kGroupFloats] [ring: ring_arrays(M) x ring_rows(M) floats].
constexpr int kHeadBytes = 1280;
constexpr int kGroupFloats = 4 * kRagThreads + kRagThreads + 48 + 2 * 2 * kRagWarps + 4;  // R, X, F0, norms, max
// (CTA-wide items use all of R, X, F0; team t uses its third of each.)
constexpr int kSmemBudget = 232448;  // 227 KB, the opt-in maximum of sm_100-class GPUs
__host__ __device__ constexpr int ring_arrays(int mode) { return mode == kPlain || one_correction(mode) ? 4 : 6; }
__host__ __device__ constexpr int ring_rows(int mode) {
  return ((kSmemBudget - kHeadBytes - 4 * kGroupFloats) / (4 * ring_arrays(mode))) & ~255;
}
// The ring is the destination of bulk copies: its start (and every array's)
// must be 16-byte aligned.
static_assert((kHeadBytes + 4 * kGroupFloats) % 16 == 0, "ring start 16-byte aligned");
constexpr size_t rag_smem_bytes(int mode) {
  return (size_t)kHeadBytes + 4 * (size_t)kGroupFloats + 4 * (size_t)ring_arrays(mode) * ring_rows(mode);
}
static_assert(ring_rows(kPlain) >= 13568 && ring_rows(kRefineDF) >= 8960, "ring sizes");
static_assert(kBigScratchRows <= ring_rows(kRefineDF), "BIG scratch fits the ring");
constexpr int kMaxStagedRows = ring_rows(kPlain);

struct RagItem {
  int kind;
  int count;  // systems in the item
  int first;  // index into the plan's system list
  int rows;   // ring rows the item occupies (padded, per array)
};

// Plan buffer on the device: [reserved (64 B)] [items] [system list].
struct RagSys {
  long off;  // first row of the system
  int n;     // rows
  int pad;
};

struct RagParams {
  const float* a;
  const float* b;
  const float* c;
  const float* d;
  float* x;                  // plain mode: FP32 solution
  double* x64;               // refined modes: FP64 solution
  float* wxh;                // refined modes, BIG systems: x (two words per row) and r, per row
  float* wxl;
  float* wr;
  unsigned long long* rel;   // refined modes: max relative residual (bits of a non-negative double)
  const RagItem* items;
  const RagSys* sys;
  int nitems;
  int sweeps;
  unsigned* status;
};

struct RagSlot {  // descriptor of an item in flight, written by the producer warp
  long off[kMaxItemSystems];  // first row of each system in the batch
  int n[kMaxItemSystems];     // rows of each system
  int base[kMaxItemSystems];  // ring row of each system's first row
  int kind;
  int count;  // systems in the item
  int rbase;  // first ring row of the item
  int rrows;  // ring rows it holds
};
constexpr int kRestageBars = kRagWarps + kTeams + 1;  // one per warp, per team, and the CTA's
static_assert(2 * kSlots * 8 + kSlots * sizeof(RagSlot) + 8 * kRestageBars <= kHeadBytes, "head fits");

__device__ __forceinline__ int odd_ceil_dev(int v) { return (v & 1) ? v : v + 1; }

// Named barrier over `count` threads with a runtime id (1 = all consumers,
// 2.. = MULTI4 groups).
__device__ __forceinline__ void group_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// Barrier of a solve group: the warp itself (gt == 32) or its named barrier.
__device__ __forceinline__ void gsync(int bar, int gt) {
  if (gt == 32)
    __syncwarp();
  else
    group_sync(bar, gt);
}

// ---------------------------------------------------------------------------
// Extended-precision helpers of the refined modes.

// x_i of the refined modes lives in two float words per row:
//   RES_DF:   (hi, lo), x = hi + lo, |lo| <= ulp(hi) / 2
//   RES_FP64: the low and high 32 bits of the double
template <int MODE>
struct XStore {
  float* h;
  float* l;
  __device__ __forceinline__ double get64(int i) const {
    if constexpr (MODE == kRefineFP64)
      return __hiloint2double(__float_as_int(l[i]), __float_as_int(h[i]));
    else
      return df_to_double(h[i], l[i]);
  }
  __device__ __forceinline__ void set64(int i, double v) {
    h[i] = __int_as_float(__double2loint(v));
    l[i] = __int_as_float(__double2hiint(v));
  }
  // x_i = v (first solve)
  __device__ __forceinline__ void init(int i, float v) {
    if constexpr (MODE == kRefineFP64) {
      set64(i, f2d_exact(v));
    } else {
      h[i] = v;
      l[i] = 0.f;
    }
  }
  // x_i += v (correction)
  __device__ __forceinline__ void add(int i, float v) {
    if constexpr (MODE == kRefineFP64) {
      set64(i, get64(i) + f2d_exact(v));
    } else {
      const float2 x = df_add(make_float2(h[i], l[i]), v);
      h[i] = x.x;
      l[i] = x.y;
    }
  }
  // r_i = d - a x_{i-1} - b x_i - c x_{i+1}, rounded to float (a = 0 at
  // i = 0, c = 0 at i = n - 1, as in the gold solver).
  __device__ __forceinline__ float residual(int i, int n, float a, float b, float c, float d) const {
    if constexpr (MODE == kRefineFP64) {
      double r = fma(-f2d_exact(b), get64(i), f2d_exact(d));
      if (i > 0) r = fma(-f2d_exact(a), get64(i - 1), r);
      if (i < n - 1) r = fma(-f2d_exact(c), get64(i + 1), r);
      return (float)r;
    } else {
      const float2 xm = i > 0 ? make_float2(h[i - 1], l[i - 1]) : make_float2(0.f, 0.f);
      const float2 xp = i < n - 1 ? make_float2(h[i + 1], l[i + 1]) : make_float2(0.f, 0.f);
      return df_residual(i > 0 ? a : 0.f, b, i < n - 1 ? c : 0.f, d, xm, make_float2(h[i], l[i]), xp);
    }
  }
};

// Adds (rr, dd) over a solve group, and its leader folds sqrt(rr) / sqrt(dd)
// into the CTA's maximum `rel` (shared memory; the kernel folds it into the
// batch maximum once at the end).  The sums stay in FP32, like the per-lane
// partials (GB300's FP64 adds, square roots and divisions are slow): enough
// for a residual check, and valid while the squares stay in FP32's range
// (|d| and |d - Tx| above ~1e-19 where not zero).  red: 2 floats per warp.
__device__ __forceinline__ void group_rel_max(float rr, float dd, int gt, int bar, int gtid, float* red,
                                              unsigned long long* rel) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_down_sync(kFull, rr, o);
    dd += __shfl_down_sync(kFull, dd, o);
  }
  if (gt > 32) {
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      red[2 * w] = rr;
      red[2 * w + 1] = dd;
    }
    group_sync(bar, gt);
    if (gtid == 0) {
      for (int q = 1; q < gt / 32; ++q) {
        rr += red[2 * (w + q)];
        dd += red[2 * (w + q) + 1];
      }
    }
  }
  if (gtid == 0) {
    const float v = dd > 0.f ? sqrtf(rr) / sqrtf(dd) : sqrtf(rr);
    atomicMax(rel, (unsigned long long)__double_as_longlong((double)v));  // the CTA's maximum, in shared memory
  }
}

// ---------------------------------------------------------------------------
// One system of n rows (ring arrays sa..sd, overwritten) solved by a group of
// gt threads (thread gtid of the group; gt == 32: one warp, else the named
// barrier `bar` over the group): chunk elimination in place, the gt
// separators solved by PCR in warp shuffles (gt == 32) or by one warp of the
// group (warp_solve_rows over shared memory R: 4*gt floats, X: gt, F0:
// 3*(gt/32)), back substitution; emit(i, x_i) for every row.
// Emit tag: x_i written over the ring's d_i.
struct EmitOverD {};

// The m = 32 q rows held in R (a, b, c, d at R, R + m, R + 2m, R + 3m; q
// odd, so the lanes' strided accesses are conflict-free) solved by one warp
// into X: lane l eliminates rows [l q, l q + q) in place, the 32 lane
// separators are solved by PCR over shuffles, then each lane substitutes
// back.  A team's separator system (m = 160) solved this way costs a few
// hundred instructions of one warp instead of log2(m) barrier-separated PCR
// steps of every thread of the team.
__device__ __forceinline__ void warp_solve_rows(float* R, float* X, int m, int lane) {
  const int q = m >> 5;
  float* ra = R + lane * q;
  float* rb = ra + m;
  float* rc = rb + m;
  float* rd = rc + m;
  ChunkSummary<float> cs;
  chunk_eliminate_smem<float>(cs, q, lane == 0, lane == 31, ra, rb, rc, rd);
  const float nD = __shfl_down_sync(kFull, cs.fD, 1);
  const float nC = __shfl_down_sync(kFull, cs.fC, 1);
  const float nA = __shfl_down_sync(kFull, cs.fA, 1);
  const float sj = warp_pcr32<float>(separator_row_s<float>(cs, nD, nC, nA));
  float sl = __shfl_up_sync(kFull, sj, 1);
  if (lane == 0) sl = 0.f;
  float* xl = X + lane * q;
  auto em = [&](int i, float v) { xl[i] = v; };
  chunk_back_smem<float>(q, sj, sl, ra, rc, rd, em);
}

// A system's right-hand side seen from the chunk starting at row r0 (chunk
// row i is system row r0 + i).
template <class Rhs>
struct ChunkRhs {
  const Rhs& rhs;
  int r0;
  static constexpr bool kPairs = Rhs::kPairs;
  __device__ __forceinline__ float operator()(int i, float a, float b, float c, float d) const {
    return rhs(r0 + i, a, b, c, d);
  }
  __device__ __forceinline__ float2 pair(int i, float a0, float b0, float c0, float d0, float a1, float b1, float c1,
                                         float d1) const {
    return rhs.pair(r0 + i, a0, b0, c0, d0, a1, b1, c1, d1);
  }
};

template <class Emit, class Rhs = RhsStaged>
__device__ __forceinline__ void group_solve(int n, int gt, int bar, int gtid, float* sa, const float* sb, float* sc,
                                            float* sd, float* R, float* X, float* F0, Emit& emit,
                                            const Rhs& rhs = Rhs()) {
  const int lane = gtid & 31, gw = gtid >> 5;
  const int kk = odd_ceil_dev((n + gt - 1) / gt);
  const int r0 = gtid * kk;
  int kr = n - r0;
  kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
  ChunkSummary<float> cs;
  rhs.start(r0);
  chunk_eliminate_smem<float>(cs, kr, gtid == 0, r0 + kr == n && kr > 0, sa + r0, sb + r0, sc + r0, sd + r0,
                              ChunkRhs<Rhs>{rhs, r0});
  float nD = __shfl_down_sync(kFull, cs.fD, 1);
  float nC = __shfl_down_sync(kFull, cs.fC, 1);
  float nA = __shfl_down_sync(kFull, cs.fA, 1);
  float sj, sl;
  if (gt == 32) {
    sj = warp_pcr32<float>(separator_row_s<float>(cs, nD, nC, nA));
    sl = __shfl_up_sync(kFull, sj, 1);
    if (lane == 0) sl = 0.f;
  } else {
    if (lane == 0) {
      F0[gw * 3 + 0] = cs.fD; F0[gw * 3 + 1] = cs.fC; F0[gw * 3 + 2] = cs.fA;
    }
    group_sync(bar, gt);
    if (lane == 31 && gw + 1 < gt / 32) {
      nD = F0[(gw + 1) * 3 + 0]; nC = F0[(gw + 1) * 3 + 1]; nA = F0[(gw + 1) * 3 + 2];
    }
    Row<float> sr = separator_row_s<float>(cs, nD, nC, nA);
    // one warp solves the separators (gt / 32 rows per lane: 5 for a team,
    // 15 for the CTA), the others wait at the barrier: measured faster than
    // a PCR over the CTA's 480 rows in shared memory (9 steps, each two
    // barriers of all 15 warps)
    R[gtid] = sr.a; R[gt + gtid] = sr.b; R[2 * gt + gtid] = sr.c; R[3 * gt + gtid] = sr.d;
    group_sync(bar, gt);
    if (gw == 0) warp_solve_rows(R, X, gt, lane);
    group_sync(bar, gt);
    sj = X[gtid];
    sl = gtid > 0 ? X[gtid - 1] : 0.f;
  }
  if constexpr (std::is_same_v<Emit, EmitOverD>) {
    chunk_back_smem_over_d<float>(kr, sj, sl, sa + r0, sc + r0, sd + r0);
  } else {
    auto em = [&](int i, float v) { emit(r0 + i, v); };
    chunk_back_smem<float>(kr, sj, sl, sa + r0, sc + r0, sd + r0, em);
  }
  if (gt != 32) group_sync(bar, gt);  // F0 / R / X reused by the next solve
}

struct EmitStore {
  float* x;
  __device__ __forceinline__ void operator()(int i, float v) { x[i] = v; }
};

// Plain solve of one staged system by its group: x_i lands in the ring's b
// slot of row i (b is not read by the back substitution), then the group
// copies the rows out in order, so every warp store is one contiguous run.
__device__ __forceinline__ void group_solve_plain(int n, int gt, int bar, int gtid, float* sa, float* sb, float* sc,
                                                  float* sd, float* R, float* X, float* F0, float* xg) {
  EmitStore em{sb};
  group_solve(n, gt, bar, gtid, sa, sb, sc, sd, R, X, F0, em);
  gsync(bar, gt);
  for (int i = gtid; i < n; i += gt) xg[i] = sb[i];
}
// x_i = v on the first solve, x_i += v on the corrections.
template <int MODE>
struct EmitX {
  XStore<MODE> xs;
  bool first;
  __device__ __forceinline__ void operator()(int i, float v) {
    if (first)
      xs.init(i, v);
    else
      xs.add(i, v);
  }
};

// Right-hand side of a correction solve: row i's residual d - (T x)_i, for
// the rows of a chunk in order, x_{i-1} and x_i carried from the row before
// (one x load per row).
template <int MODE>
struct RhsResidual;
template <>
struct RhsResidual<kRefineDF> {
  static constexpr bool kPairs = false;
  XStore<kRefineDF> xs;
  int n;
  mutable float2 xm, x0;
  __device__ __forceinline__ float2 at(int i) const {
    return i >= 0 && i < n ? make_float2(xs.h[i], xs.l[i]) : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void start(int i) const {
    xm = at(i - 1);
    x0 = at(i);
  }
  __device__ __forceinline__ float operator()(int i, float a, float b, float c, float d) const {
    const float2 xp = at(i + 1);
    const float r = df_residual(i > 0 ? a : 0.f, b, i < n - 1 ? c : 0.f, d, xm, x0, xp);
    xm = x0;
    x0 = xp;
    return r;
  }
};
template <>
struct RhsResidual<kRefineFP64> {
  static constexpr bool kPairs = false;
  XStore<kRefineFP64> xs;
  int n;
  mutable double xm, x0;
  __device__ __forceinline__ double at(int i) const { return i >= 0 && i < n ? xs.get64(i) : 0.0; }
  __device__ __forceinline__ void start(int i) const {
    xm = at(i - 1);
    x0 = at(i);
  }
  __device__ __forceinline__ float operator()(int i, float a, float b, float c, float d) const {
    const double xp = at(i + 1);
    double r = fma(-f2d_exact(b), x0, f2d_exact(d));
    r = fma(-f2d_exact(i > 0 ? a : 0.f), xm, r);
    r = fma(-f2d_exact(i < n - 1 ? c : 0.f), xp, r);
    xm = x0;
    x0 = xp;
    return (float)r;
  }
};

// The refinement's re-staging of a system's original a, c, d into its ring
// slots (the FP32 elimination overwrote them there; b and the x words are
// untouched): a bulk copy per array on the group's own mbarrier `mb`, whose
// phase parity is bit `pbit` of `par`.  Every thread of the group orders its
// earlier ring accesses before the copy (proxy fence + group barrier); the
// leader issues; all wait (bounded).
struct Restage {
  uint64_t* mb;
  int pbit;
  float* dst_a;  // ring slot of the system's first padded row, per array
  float* dst_c;
  float* dst_d;
  const float* src_a;  // the same rows in global memory (16-byte aligned)
  const float* src_c;
  const float* src_d;
  uint32_t bytes;
  bool with_d;  // false: a and c only
};

__device__ __forceinline__ void restage(const Restage& rs, uint32_t& par, int gt, int bar, int gtid,
                                        unsigned* status) {
  fence_proxy_async_smem();
  gsync(bar, gt);
  if (gtid == 0) {
    mbar_arrive_expect_tx(rs.mb, (rs.with_d ? 3u : 2u) * rs.bytes);
    bulk_g2s(rs.dst_a, rs.src_a, rs.bytes, rs.mb);
    bulk_g2s(rs.dst_c, rs.src_c, rs.bytes, rs.mb);
    if (rs.with_d) bulk_g2s(rs.dst_d, rs.src_d, rs.bytes, rs.mb);
  }
  mbar_wait(rs.mb, (par >> rs.pbit) & 1u, status);
  par ^= 1u << rs.pbit;
}

// Refinement of one staged system by its solve group (see the file comment).
// sa..sd: the system's rows in the ring, xh / xl: its x words in the ring.
// Before each correction solve and the final residual pass the originals are
// re-staged into the ring, so the residuals read shared memory only.
template <int MODE>
__device__ __forceinline__ void group_refine(const RagParams& p, const RagSys& sy, int gt, int bar, int gtid,
                                             float* sa, const float* sb, float* sc, float* sd, float* xh, float* xl,
                                             float* R, float* X, float* F0, double* red, uint64_t* mb, int pbit,
                                             uint32_t& par) {
  const int n = sy.n;
  XStore<MODE> xs{xh, xl};
  const long lo = sy.off & ~3L, hi = (sy.off + n + 3) & ~3L;
  const int pad = (int)(sy.off - lo);
  const Restage rs{mb, pbit, sa - pad, sc - pad, sd - pad, p.a + lo, p.c + lo, p.d + lo,
                   (uint32_t)(4 * (hi - lo)), true};
  EmitX<MODE> first{xs, true};
  group_solve(n, gt, bar, gtid, sa, sb, sc, sd, R, X, F0, first);
  for (int sw = 0; sw < p.sweeps; ++sw) {
    // correction: the residual of each row formed as the row is eliminated
    restage(rs, par, gt, bar, gtid, p.status);
    EmitX<MODE> add{xs, false};
    group_solve(n, gt, bar, gtid, sa, sb, sc, sd, R, X, F0, add, RhsResidual<MODE>{xs, n});
  }
  restage(rs, par, gt, bar, gtid, p.status);
  float rr = 0.f, dd = 0.f;
  double* xo = p.x64 + sy.off;
  for (int i = gtid; i < n; i += gt) {
    const float d = sd[i];
    const float r = xs.residual(i, n, sa[i], sb[i], sc[i], d);
    rr = fmaf(r, r, rr);
    dd = fmaf(d, d, dd);
    xo[i] = xs.get64(i);
  }
  group_rel_max(rr, dd, gt, bar, gtid, reinterpret_cast<float*>(red),
                reinterpret_cast<unsigned long long*>(red + 2 * kRagWarps));
}

// Right-hand side of the one-correction modes' correction solve: row i's
// residual d - (T x0)_i for the FP32 solution x0 (held in the ring's b
// words), rows of a chunk in order, x0_{i-1} and x0_i carried.
template <int M>
struct RhsResidual1 {
  static constexpr bool kPairs = M == kRefineDF;
  const float* x0w;
  int n;
  mutable float xm, x0;
  __device__ __forceinline__ float at(int i) const { return i >= 0 && i < n ? x0w[i] : 0.f; }
  __device__ __forceinline__ void start(int i) const {
    xm = at(i - 1);
    x0 = at(i);
  }
  __device__ __forceinline__ float operator()(int i, float a, float b, float c, float d) const {
    const float xp = at(i + 1);
    a = i > 0 ? a : 0.f;
    c = i < n - 1 ? c : 0.f;
    float r;
    if constexpr (M == kRefineFP64) {
      double v = fma(-f2d_exact(b), f2d_exact(x0), f2d_exact(d));
      v = fma(-f2d_exact(a), f2d_exact(xm), v);
      v = fma(-f2d_exact(c), f2d_exact(xp), v);
      r = (float)v;
    } else {
      r = f_residual(a, b, c, d, xm, x0, xp);
    }
    xm = x0;
    x0 = xp;
    return r;
  }
  // Rows i and i + 1, both interior rows of a chunk (so 0 < i + 1 and
  // i + 2 < n: only row i's a can lie outside the system), in paired
  // instructions: residual_parts2 is residual_parts component by component.
  __device__ __forceinline__ float2 pair(int i, float a0, float b0, float c0, float d0, float a1, float b1, float c1,
                                         float d1) const {
    const float x1 = x0w[i + 1], x2 = x0w[i + 2];
    float2 s, t;
    residual_parts2(make_float2(i > 0 ? a0 : 0.f, a1), make_float2(b0, b1), make_float2(c0, c1),
                    make_float2(d0, d1), make_float2(xm, x0), make_float2(x0, x1), make_float2(x1, x2), s, t);
    xm = x1;
    x0 = x2;
    return __fadd2_rn(s, t);
  }
};

// The last pass of the one-correction modes: x = x0 + e (x0 in the ring's b
// words xw, e in its d words ew), its residual d - T x, the group's
// ||d - T x|| / ||d|| folded into the CTA's maximum, and x written as FP64.
// Rows i = gtid + q gt; the original a, b, c, d come from global memory (L2,
// coalesced across the group), each thread keeping the loads of its next
// kAhead rows in flight.  The double-float form takes its rows two at a time
// (i and i + gt) in paired FP32 instructions, the same operations as the
// scalar form component by component.
template <int M>
__device__ __forceinline__ void refine1_final(const RagParams& p, const RagSys& sy, int gt, int bar, int gtid,
                                              const float* xw, const float* ew, double* red) {
  const int n = sy.n;
  const float* ga = p.a + sy.off;
  const float* gb = p.b + sy.off;
  const float* gc = p.c + sy.off;
  const float* gd = p.d + sy.off;
  double* xo = p.x64 + sy.off;
  constexpr int kAhead = 4;  // two pairs
  float na[kAhead], nb[kAhead], nc[kAhead], nd[kAhead];
#pragma unroll
  for (int q = 0; q < kAhead; ++q) {
    const int j = gtid + q * gt;
    const bool in = j < n;
    na[q] = in ? ga[j] : 0.f;
    nb[q] = in ? gb[j] : 0.f;
    nc[q] = in ? gc[j] : 0.f;
    nd[q] = in ? gd[j] : 0.f;
  }
  float2 rr = make_float2(0.f, 0.f), dd = make_float2(0.f, 0.f);
  const auto out = [&](int i, float h0, float e0) {
    float l;
    const float h = two_sum(h0, e0, l);
    xo[i] = df_to_double(h, l);
  };
  for (int i0 = gtid; i0 < n; i0 += kAhead * gt) {
#pragma unroll
    for (int q = 0; q < kAhead; q += 2) {
      const int i = i0 + q * gt, j = i + gt;  // j > 0
      if (i >= n) break;
      const bool jin = j < n;
      float2 a = make_float2(na[q], na[q + 1]), b = make_float2(nb[q], nb[q + 1]);
      float2 c = make_float2(nc[q], nc[q + 1]), d = make_float2(nd[q], nd[q + 1]);
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int f = i + (u + kAhead) * gt;
        if (f < n) {
          na[q + u] = ga[f];
          nb[q + u] = gb[f];
          nc[q + u] = gc[f];
          nd[q + u] = gd[f];
        }
      }
      if (i == 0) a.x = 0.f;
      if (i == n - 1) c.x = 0.f;
      if (j >= n - 1) c.y = 0.f;
      // x words of rows i - 1, i, i + 1 and j - 1, j, j + 1 (zero outside the system)
      const float2 xmh = make_float2(i > 0 ? xw[i - 1] : 0.f, jin ? xw[j - 1] : 0.f);
      const float2 xml = make_float2(i > 0 ? ew[i - 1] : 0.f, jin ? ew[j - 1] : 0.f);
      const float2 x0h = make_float2(xw[i], jin ? xw[j] : 0.f);
      const float2 x0l = make_float2(ew[i], jin ? ew[j] : 0.f);
      const float2 xph = make_float2(i + 1 < n ? xw[i + 1] : 0.f, j + 1 < n ? xw[j + 1] : 0.f);
      const float2 xpl = make_float2(i + 1 < n ? ew[i + 1] : 0.f, j + 1 < n ? ew[j + 1] : 0.f);
      float2 r;
      if constexpr (M == kRefineFP64) {
        const auto x64 = [](float h0, float e0) {
          float l;
          const float h = two_sum(h0, e0, l);
          return df_to_double(h, l);
        };
        const auto res = [&](float a1, float b1, float c1, float d1, double m1, double z1, double p1) {
          double v = fma(-f2d_exact(b1), z1, f2d_exact(d1));
          v = fma(-f2d_exact(a1), m1, v);
          v = fma(-f2d_exact(c1), p1, v);
          return (float)v;
        };
        r.x = res(a.x, b.x, c.x, d.x, x64(xmh.x, xml.x), x64(x0h.x, x0l.x), x64(xph.x, xpl.x));
        r.y = jin ? res(a.y, b.y, c.y, d.y, x64(xmh.y, xml.y), x64(x0h.y, x0l.y), x64(xph.y, xpl.y)) : 0.f;
      } else {
        r = df_residual2(a, b, c, d, xmh, xml, x0h, x0l, xph, xpl);
      }
      if (!jin) {  // no row j: its prefetch registers may hold an earlier row
        r.y = 0.f;
        d.y = 0.f;
      }
      rr = __ffma2_rn(r, r, rr);
      dd = __ffma2_rn(d, d, dd);
      out(i, x0h.x, x0l.x);
      if (jin) out(j, x0h.y, x0l.y);
    }
  }
  group_rel_max(rr.x + rr.y, dd.x + dd.y, gt, bar, gtid, reinterpret_cast<float*>(red),
                reinterpret_cast<unsigned long long*>(red + 2 * kRagWarps));
}

// One-correction refinement (sweeps == 1) of one staged system by its solve
// group, in the ring's four arrays: the FP32 solve leaves x0 in the b words;
// a, c, d are re-staged; the correction solve (b read from global memory,
// each row's residual formed as the row is eliminated) leaves its solution e
// in the d words; a and c are re-staged once more, and the final pass forms
// d - T (x0 + e) with b and d from global memory, folds its norm into the
// CTA's maximum and writes x0 + e as FP64.  M: kRefineDF or kRefineFP64.
template <int M>
__device__ __forceinline__ void group_refine1(const RagParams& p, const RagSys& sy, int gt, int bar, int gtid,
                                              float* sa, float* sb, float* sc, float* sd, float* R, float* X,
                                              float* F0, double* red, uint64_t* mb, int pbit, uint32_t& par) {
  const int n = sy.n;
  const long lo = sy.off & ~3L, hi = (sy.off + n + 3) & ~3L;
  const int pad = (int)(sy.off - lo);
  const uint32_t bytes = (uint32_t)(4 * (hi - lo));
  const float* gb = p.b + sy.off;
  EmitStore to_b{sb};
  group_solve(n, gt, bar, gtid, sa, sb, sc, sd, R, X, F0, to_b);
  restage(Restage{mb, pbit, sa - pad, sc - pad, sd - pad, p.a + lo, p.c + lo, p.d + lo, bytes, true}, par, gt, bar,
          gtid, p.status);
  EmitOverD to_d;
  group_solve(n, gt, bar, gtid, sa, gb, sc, sd, R, X, F0, to_d, RhsResidual1<M>{sb, n});
  if (gt == 32) __syncwarp();  // the e words are complete (group_solve ends on the barrier otherwise)
  refine1_final<M>(p, sy, gt, bar, gtid, sb, sd, red);
}

// A BIG system (rows read straight from global memory, right-hand side rhs):
// kBigSepRows chunks, kBigChunks per consumer thread; their separators solved
// by PCR across the consumers in shared memory, then every chunk eliminated
// again and substituted back, emit(i, x_i).  Scratch: separator rows Ra..Rd,
// their solution Xs, the chunks' first-row coefficients FD, FC, FA (kBigSepRows
// floats each).
template <class Emit>
__device__ __forceinline__ void solve_big(const RagSys& sy, const float* __restrict__ ga,
                                          const float* __restrict__ gb, const float* __restrict__ gc,
                                          const float* __restrict__ gd, int tid, float* Ra, float* Rb, float* Rc,
                                          float* Rd, float* Xs, float* FD, float* FC, float* FA, Emit& emit) {
  const int n = sy.n;
  constexpr int KC = kBigKC;
  constexpr int NS = kBigSepRows;
  const int kk = odd_ceil_dev((n + NS - 1) / NS);
  // pass 1: eliminate every chunk; export its first-row coefficients and the
  // part of its separator row that needs no neighbour
#pragma unroll 1
  for (int q = 0; q < kBigChunks; ++q) {
    const int j = q * kRagThreads + tid;
    const int r0 = j * kk;
    int kr = n - r0;
    kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
    Chunk<float, KC> ch;
    chunk_eliminate<float, KC>(ch, kr, j == 0, r0 + kr == n && kr > 0, ga + r0, gb + r0, gc + r0, gd + r0);
    FD[j] = ch.fD; FC[j] = ch.fC; FA[j] = ch.fA;
    const Row<float>& e = ch.sep;
    Ra[j] = -e.a * ch.lA; Rb[j] = e.b - e.a * ch.lC; Rc[j] = e.c; Rd[j] = e.d - e.a * ch.lD;
  }
  consumer_sync(kRagThreads);
  // separator rows (the next chunk's first row folded in); PCR over all NS
  Row<float> sr[kBigChunks];
#pragma unroll
  for (int q = 0; q < kBigChunks; ++q) {
    const int j = q * kRagThreads + tid;
    const float nD = j + 1 < NS ? FD[j + 1] : 0.f;
    const float nC = j + 1 < NS ? FC[j + 1] : 0.f;
    const float nA = j + 1 < NS ? FA[j + 1] : 0.f;
    const float ec = Rc[j];
    sr[q] = Row<float>{Ra[j], Rb[j] - ec * nA, -ec * nC, Rd[j] - ec * nD};
  }
  consumer_sync(kRagThreads);  // every partial row read before PCR overwrites them
  const Row<float> id{0.f, 1.f, 0.f, 0.f};
  for (int dl = 1; dl < NS; dl *= 2) {
#pragma unroll
    for (int q = 0; q < kBigChunks; ++q) {
      const int j = q * kRagThreads + tid;
      Ra[j] = sr[q].a; Rb[j] = sr[q].b; Rc[j] = sr[q].c; Rd[j] = sr[q].d;
    }
    consumer_sync(kRagThreads);
#pragma unroll
    for (int q = 0; q < kBigChunks; ++q) {
      const int j = q * kRagThreads + tid;
      const Row<float> L = j >= dl ? Row<float>{Ra[j - dl], Rb[j - dl], Rc[j - dl], Rd[j - dl]} : id;
      const Row<float> R = j + dl < NS ? Row<float>{Ra[j + dl], Rb[j + dl], Rc[j + dl], Rd[j + dl]} : id;
      sr[q] = reduce_row(sr[q], L, R);
    }
    consumer_sync(kRagThreads);
  }
#pragma unroll
  for (int q = 0; q < kBigChunks; ++q) Xs[q * kRagThreads + tid] = tdiv(sr[q].d, sr[q].b);
  consumer_sync(kRagThreads);
  // pass 2: eliminate again and substitute back
#pragma unroll 1
  for (int q = 0; q < kBigChunks; ++q) {
    const int j = q * kRagThreads + tid;
    const int r0 = j * kk;
    int kr = n - r0;
    kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
    Chunk<float, KC> ch;
    chunk_eliminate<float, KC>(ch, kr, j == 0, r0 + kr == n && kr > 0, ga + r0, gb + r0, gc + r0, gd + r0);
    auto em = [&](int i, float v) { emit(r0 + i, v); };
    chunk_back_emit<float, KC>(ch, kr, Xs[j], j > 0 ? Xs[j - 1] : 0.f, em);
  }
  consumer_sync(kRagThreads);  // scratch reused by the next solve
}

// Refinement of a BIG system by the whole CTA; x and r in the global scratch.
template <int MODE>
__device__ __forceinline__ void big_refine(const RagParams& p, const RagSys& sy, int tid, float* Ra, float* Rb,
                                           float* Rc, float* Rd, float* Xs, float* FD, float* FC, float* FA,
                                           double* red) {
  const int n = sy.n;
  const float* ga = p.a + sy.off;
  const float* gb = p.b + sy.off;
  const float* gc = p.c + sy.off;
  const float* gd = p.d + sy.off;
  float* wr = p.wr + sy.off;
  XStore<MODE> xs{p.wxh + sy.off, p.wxl + sy.off};
  for (int sw = -1; sw < p.sweeps; ++sw) {  // sw = -1: the first solve
    if (sw >= 0) {
      for (int i = tid; i < n; i += kRagThreads) wr[i] = xs.residual(i, n, ga[i], gb[i], gc[i], gd[i]);
      consumer_sync(kRagThreads);
    }
    EmitX<MODE> em{xs, sw < 0};
    solve_big(sy, ga, gb, gc, sw < 0 ? gd : wr, tid, Ra, Rb, Rc, Rd, Xs, FD, FC, FA, em);
  }
  float rr = 0.f, dd = 0.f;
  double* xo = p.x64 + sy.off;
  for (int i = tid; i < n; i += kRagThreads) {
    const float d = gd[i];
    const float r = xs.residual(i, n, ga[i], gb[i], gc[i], d);
    rr = fmaf(r, r, rr);
    dd = fmaf(d, d, dd);
    xo[i] = xs.get64(i);
  }
  group_rel_max(rr, dd, kRagThreads, 1, tid, reinterpret_cast<float*>(red),
                reinterpret_cast<unsigned long long*>(red + 2 * kRagWarps));
  consumer_sync(kRagThreads);
}

// ---------------------------------------------------------------------------
// BIG: the kernel carries the BIG-item path.  Its register demand (kBigChunks
// chunk states per thread) would set the allocation of the whole kernel and
// push values of the other items' solve loops into local memory, so plans
// without BIG items run the kernel compiled without it.
template <int MODE, bool BIG>
__global__ void __launch_bounds__(kRagThreads + 32, 1) ragged_kernel(RagParams p) {
  static_assert((kRagThreads + 32) % 128 == 0, "16 warps: 4 per SM sub-partition");
  constexpr int RR = ring_rows(MODE);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + kSlots;
  RagSlot* desc = reinterpret_cast<RagSlot*>(smem + 2 * kSlots * 8);
  uint64_t* rbar = reinterpret_cast<uint64_t*>(smem + 2 * kSlots * 8 + kSlots * sizeof(RagSlot));  // restaging
  float* Rsh = reinterpret_cast<float*>(smem + kHeadBytes);  // group / CTA separators: 4 x kRagThreads
  float* Xsh = Rsh + 4 * kRagThreads;                           // their solution
  float* F0 = Xsh + kRagThreads;                                // lane-0 first-row coefficients (3 per warp)
  double* red = reinterpret_cast<double*>(F0 + 48);             // norms: 2 per warp
  unsigned long long* cta_rel = reinterpret_cast<unsigned long long*>(red + 2 * kRagWarps);  // the CTA's max
  float* ring = Rsh + kGroupFloats;                             // array q at ring + q * RR
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    for (int s = 0; s < kSlots; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kRagWarps);
    }
    for (int q = 0; q < kRestageBars; ++q) mbar_init(&rbar[q], 1);
    mbar_fence_init();
    *cta_rel = 0ull;
  }
  __syncthreads();

  if (tid >= kRagThreads) {  // ---------------- producer warp ----------------
    // Every lane runs the same control flow; lane q handles system q of an
    // item (its descriptor entry and its four bulk copies), lane 0 the
    // item-wide fields and the arrive.
    int k = 0;       // items published
    int oldest = 0;  // oldest item not yet reclaimed
    int head = 0;    // next free ring row
    int ends = 0;    // END markers published: one per team
    RagItem nxt{kEnd, 0, 0, 0};
    if ((int)blockIdx.x < p.nitems) nxt = p.items[blockIdx.x];
    // item records and the lanes' system records are loaded one item ahead
    RagSys nsy{0, 0, 0};
    if (nxt.kind != kEnd && lane < nxt.count) nsy = p.sys[nxt.first + lane];
    for (int item = blockIdx.x;; item += gridDim.x) {
      const bool end = item >= p.nitems;
      const RagItem it = nxt;
      const RagSys sy = end ? RagSys{0, 0, 0} : nsy;
      if (item + (int)gridDim.x < p.nitems) {
        nxt = p.items[item + gridDim.x];
        if (lane < nxt.count) nsy = p.sys[nxt.first + lane];
      }
      int kind = end ? (int)kEnd : it.kind;
      if (kind == kSingle && it.rows > RR) kind = kBig;  // does not fit this mode's ring
      // ring rows of this lane's system and their exclusive prefix over lanes
      const long lo = sy.off & ~3L, hi = (sy.off + sy.n + 3) & ~3L;
      const int mine = (!end && kind != kBig && lane < it.count) ? (int)(hi - lo) : 0;
      int pre = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(kFull, pre, o);
        if (lane >= o) pre += v;
      }
      const int need = end ? 0 : (kind == kBig ? kBigScratchRows : __shfl_sync(kFull, pre, 31));
      pre -= mine;
      // a free slot and `need` contiguous ring rows, reclaiming oldest first
      int place = -1;
      bool ok = true;
      while (true) {
        const int inflight = k - oldest;
        if (inflight == 0) {
          head = 0;
          place = 0;
          break;
        }
        if (inflight < kSlots) {
          const int tail = desc[oldest % kSlots].rbase;
          if (tail < head) {  // occupied [tail, head)
            if (head + need <= RR) { place = head; break; }
            if (need <= tail) { place = 0; break; }
          } else if (head + need <= tail) {  // occupied [tail, RR) and [0, head)
            place = head;
            break;
          }
        }
        // lane 0 waits (bounded); the verdict is the warp's, and every lane
        // then acquires the completed phase itself
        bool w = true;
        if (lane == 0) w = mbar_wait(&empty[oldest % kSlots], (oldest / kSlots) & 1, p.status);
        if (!__shfl_sync(kFull, (int)w, 0)) {
          ok = false;
          break;
        }
        mbar_try_wait(&empty[oldest % kSlots], (oldest / kSlots) & 1);
        ++oldest;
      }
      if (!ok) break;  // consumers time out on their own waits
      const int s = k % kSlots;
      __syncwarp();  // every lane has read desc[oldest].rbase before slot s is rewritten
      if (lane < (end ? 0 : it.count)) {
        desc[s].off[lane] = sy.off;
        desc[s].n[lane] = sy.n;
        desc[s].base[lane] = kind == kBig ? place : place + pre + (int)(sy.off - lo);
      }
      if (lane == 0) {
        desc[s].kind = kind;
        desc[s].count = end ? 0 : it.count;
        desc[s].rbase = place;
        desc[s].rrows = need;
      }
      __syncwarp();  // the descriptor is complete before lane 0 publishes it
      if (lane == 0) {
        // bytes of the whole item in the one arrive: the phase cannot
        // complete before every copy has landed
        if (end || kind == kBig)
          mbar_arrive(&full[s]);
        else
          mbar_arrive_expect_tx(&full[s], 16u * (uint32_t)need);
      }
      if (end) {
        head = place;
        ++k;
        if (++ends == kTeams) break;
        continue;
      }
      __syncwarp();
      if (mine > 0) {
        const uint32_t bytes = 4u * (uint32_t)mine;
        const int cur = place + pre;
        bulk_g2s(ring + 0 * RR + cur, p.a + lo, bytes, &full[s]);
        bulk_g2s(ring + 1 * RR + cur, p.b + lo, bytes, &full[s]);
        bulk_g2s(ring + 2 * RR + cur, p.c + lo, bytes, &full[s]);
        bulk_g2s(ring + 3 * RR + cur, p.d + lo, bytes, &full[s]);
      }
      head = place + need;
      ++k;
    }
    return;
  }

  // ---------------- consumers ----------------
  // Phase 1: the CTA's SINGLE and BIG items (the plan puts them first), all
  // 15 warps on each.  Phase 2, from the first team item on: team t (warps
  // 5t .. 5t+4, named barrier 2 + t) takes items k0 + t, k0 + t + 3, ...
  // and releases each with 3 arrivals per warp, so every slot's empty
  // barrier still completes after 15.
  float* A = ring;  // the consumers overwrite a, c, d (and, plain, b with x) of a staged item in place
  float* B = ring + RR;
  float* C = ring + 2 * RR;
  float* D = ring + 3 * RR;
  float* XH = ring + 4 * RR;  // refined modes: x words
  float* XL = ring + 5 * RR;
  uint32_t rpar = 0;  // phase parities of the restaging barriers this thread uses
  auto consume = [&]() {
    int k = 0;
    for (;; ++k) {
      const int s = k % kSlots;
      const bool ok = consumer_sync_and(kRagThreads, mbar_wait(&full[s], (k / kSlots) & 1, p.status));
      if (!ok) return;
      const RagSlot& ds = desc[s];
      const int kind = ds.kind;
      if (kind == kMulti || kind == kGroup) break;  // the team phase starts at item k
      if (kind == kEnd) return;
      const RagSys sy{ds.off[0], ds.n[0], 0};
      if (kind == kSingle) {
        const int base = ds.base[0];
        if constexpr (MODE == kPlain) {
          group_solve_plain(sy.n, kRagThreads, 1, tid, A + base, B + base, C + base, D + base, Rsh, Xsh, F0,
                            p.x + sy.off);
        } else if constexpr (one_correction(MODE)) {
          group_refine1<residual_mode(MODE)>(p, sy, kRagThreads, 1, tid, A + base, B + base, C + base, D + base,
                                             Rsh, Xsh, F0, red, &rbar[kRagWarps + kTeams], kRagWarps + kTeams, rpar);
        } else {
          group_refine<MODE>(p, sy, kRagThreads, 1, tid, A + base, B + base, C + base, D + base, XH + base, XL + base,
                             Rsh, Xsh, F0, red, &rbar[kRagWarps + kTeams], kRagWarps + kTeams, rpar);
        }
      } else if constexpr (!BIG) {  // the host launches this form only for plans without BIG items
        record_error(p.status, TRIDI_DEVERR_BAD_PLAN);
      } else {  // kBig
        const int rb = ds.rbase;
        float* Ra = A + rb;
        float* Rb = B + rb;
        float* Rc = C + rb;
        float* Rd = D + rb;
        if constexpr (MODE == kPlain) {
          EmitStore em{p.x + sy.off};
          solve_big(sy, p.a + sy.off, p.b + sy.off, p.c + sy.off, p.d + sy.off, tid, Ra, Rb, Rc, Rd,
                    Ra + kBigSepRows, Rb + kBigSepRows, Rc + kBigSepRows, Rd + kBigSepRows, em);
        } else {
          big_refine<residual_mode(MODE)>(p, sy, tid, Ra, Rb, Rc, Rd, Ra + kBigSepRows, Rb + kBigSepRows,
                                          Rc + kBigSepRows, Rd + kBigSepRows, red);
        }
      }
      release_stage(&empty[s]);
    }
    const int team = warp / kTeamWarps, tw = warp - team * kTeamWarps;
    const int ttid = tid - team * kTeamThreads, tbar = 2 + team;
    float* tR = Rsh + team * 4 * kTeamThreads;
    float* tX = Xsh + team * kTeamThreads;
    float* tF = F0 + team * 3 * kTeamWarps;
    for (k += team;; k += kTeams) {
      const int s = k % kSlots;
      const bool ok = named_sync_and(tbar, kTeamThreads, mbar_wait(&full[s], (k / kSlots) & 1, p.status));
      if (!ok) return;
      const RagSlot& ds = desc[s];
      const int kind = ds.kind;
      if (kind == kEnd) return;
      if (kind == kMulti) {
        if (tw < ds.count) {
          const RagSys sy{ds.off[tw], ds.n[tw], 0};
          const int base = ds.base[tw];
          if constexpr (MODE == kPlain) {
            group_solve_plain(sy.n, 32, 0, lane, A + base, B + base, C + base, D + base, nullptr, nullptr, nullptr,
                              p.x + sy.off);
          } else if constexpr (one_correction(MODE)) {
            group_refine1<residual_mode(MODE)>(p, sy, 32, 0, lane, A + base, B + base, C + base, D + base, nullptr,
                                               nullptr, nullptr, red, &rbar[warp], warp, rpar);
          } else {
            group_refine<MODE>(p, sy, 32, 0, lane, A + base, B + base, C + base, D + base, XH + base, XL + base,
                               nullptr, nullptr, nullptr, red, &rbar[warp], warp, rpar);
          }
        }
      } else if (kind == kGroup) {
        const RagSys sy{ds.off[0], ds.n[0], 0};
        const int base = ds.base[0];
        if constexpr (MODE == kPlain) {
          group_solve_plain(sy.n, kTeamThreads, tbar, ttid, A + base, B + base, C + base, D + base, tR, tX, tF,
                            p.x + sy.off);
        } else if constexpr (one_correction(MODE)) {
          group_refine1<residual_mode(MODE)>(p, sy, kTeamThreads, tbar, ttid, A + base, B + base, C + base, D + base,
                                             tR, tX, tF, red, &rbar[kRagWarps + team], kRagWarps + team, rpar);
        } else {
          group_refine<MODE>(p, sy, kTeamThreads, tbar, ttid, A + base, B + base, C + base, D + base, XH + base,
                             XL + base, tR, tX, tF, red, &rbar[kRagWarps + team], kRagWarps + team, rpar);
        }
      } else {
        record_error(p.status, TRIDI_DEVERR_BAD_PLAN);  // a CTA-wide item after the team phase began
        return;
      }
      release_stage_n(&empty[s], kTeams);
    }
  };
  consume();
  if constexpr (MODE != kPlain) {  // every consumer has left its loop: fold the CTA's maximum in once
    consumer_sync(kRagThreads);
    if (tid == 0) atomicMax(p.rel, *cta_rel);
  }
}

// ---------------------------------------------------------------------------
// Host plan.
struct RaggedPlan {
  std::vector<RagItem> items;
  std::vector<RagSys> sys;
  long total_rows = 0;
  int num_systems = 0;
  bool has_big = false;     // an item of kind kBig
  int max_single_rows = 0;  // ring rows of the largest SINGLE item
  // BIG items in a launch whose ring holds `ring_rows` rows per array (a
  // SINGLE item beyond it is solved as BIG)
  bool needs_big(int ring_rows) const { return has_big || max_single_rows > ring_rows; }
  size_t device_bytes() const {
    return 64 + items.size() * sizeof(RagItem) + sys.size() * sizeof(RagSys);
  }
};

namespace {
long padded_rows(long off, int n) { return ((off + n + 3) & ~3L) - (off & ~3L); }
}  // namespace

long ragged_team_max_rows() { return ring_rows(kRefineDF); }

}  // namespace tridi

using tridi::RaggedPlan;

namespace tridi {
namespace {
tridi_status plan_create(const long* offsets, int num_systems, bool refine, void** plan_out);
}  // namespace
}  // namespace tridi

extern "C" {

tridi_status tridi_ragged_plan_create(const long* offsets, int num_systems, void** plan_out) {
  return tridi::plan_create(offsets, num_systems, false, plan_out);
}

tridi_status tridi_ragged_plan_create_refine(const long* offsets, int num_systems, void** plan_out) {
  return tridi::plan_create(offsets, num_systems, true, plan_out);
}

}  // extern "C"

namespace tridi {
namespace {
// The work list of a plan (see the file comment); refine: threads per system
// from the refinement's tuning table where it has an entry.
tridi_status plan_create(const long* offsets, int num_systems, bool refine, void** plan_out) {
  if (!offsets || num_systems <= 0 || !plan_out) return TRIDI_ERROR_INVALID_VALUE;
  auto* plan = new RaggedPlan();
  plan->num_systems = num_systems;
  plan->total_rows = offsets[num_systems];
  std::vector<int> order(num_systems);
  for (int s = 0; s < num_systems; ++s) {
    const long n = offsets[s + 1] - offsets[s];
    if (n <= 0 || n > kMaxBigRows) {
      delete plan;
      return TRIDI_ERROR_UNSUPPORTED_SIZE;
    }
    order[s] = s;
  }
  // largest systems first: they are the longest items (longest-processing-time order)
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return offsets[x + 1] - offsets[x] > offsets[y + 1] - offsets[y];
  });
  plan->sys.reserve(num_systems);
  for (int s : order) plan->sys.push_back(RagSys{offsets[s], (int)(offsets[s + 1] - offsets[s]), 0});
  // threads per system: the autotuned choice for the system's size bucket,
  // else 32 up to 480 rows, 160 up to 4800, the whole CTA above
  auto threads_for = [refine](long n) {
    int t = refine ? tuned(TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS, ilog2(n)) : 0;
    if (t == 0) t = tuned(TRIDI_AUTOTUNE_RAGGED_THREADS, ilog2(n));
    if (t == 32 || t == kTeamThreads || t == kRagThreads) return t;
    return n <= kWarpMaxRows ? 32 : (n <= kGroupMaxRows ? kTeamThreads : kRagThreads);
  };
  const long kPackCap = ragged_team_max_rows();  // a team item fits the ring of every mode
  std::vector<RagItem> cta_items, team_items;      // CTA-wide items go first (phase 1 of the kernel)
  int i = 0;
  while (i < num_systems) {
    const RagSys& sy = plan->sys[i];
    const long pr = padded_rows(sy.off, sy.n);
    if (pr > kMaxStagedRows) {
      cta_items.push_back(RagItem{(int)kBig, 1, i, 0});
      ++i;
      continue;
    }
    const int th = pr > kPackCap ? kRagThreads : threads_for(sy.n);
    if (th == kRagThreads) {
      cta_items.push_back(RagItem{(int)kSingle, 1, i, (int)pr});
      ++i;
      continue;
    }
    if (th == kTeamThreads) {
      team_items.push_back(RagItem{(int)kGroup, 1, i, (int)pr});
      ++i;
      continue;
    }
    RagItem it{(int)kMulti, 0, i, 0};
    while (i < num_systems && it.count < kMaxItemSystems) {
      const RagSys& t = plan->sys[i];
      const long tr = padded_rows(t.off, t.n);
      if (tr > kPackCap || threads_for(t.n) != 32 || it.rows + tr > kPackCap) break;
      it.rows += (int)tr;
      ++it.count;
      ++i;
    }
    team_items.push_back(it);
  }
  // Plain solves: CTA b takes the list's items b, b + G, b + 2G, ... (G = the
  // launch's CTAs), so every run of G consecutive items gives each CTA one.
  // The team items go in such rounds of the size order interleaved from both
  // ends -- largest round, smallest, second largest, ... -- so each CTA's
  // teams alternate large and small items and its ring holds fewer large ones
  // at a time (100000-system batch: 0.679 -> 0.636 ms).  A last, partial round
  // stays last, keeping the rounds before it aligned with the CTAs.  The
  // refinement, bound by its arithmetic rather than by the ring, keeps the
  // largest-first order (interleaved: 1.81 -> 1.93 ms).
  const DeviceInfo* dev = refine ? nullptr : current_device();
  const long nall = (long)(cta_items.size() + team_items.size());
  const long G = dev ? std::min<long>(dev->sm_count, nall) : 0;
  if (G > 0 && (long)team_items.size() >= 2 * G && tunable(TRIDI_TUNE_RAGGED_ORDER) != 2) {
    const long R = (long)team_items.size() / G;  // full rounds
    std::vector<RagItem> mixed;
    mixed.reserve(team_items.size());
    const auto round = [&](long r) {
      mixed.insert(mixed.end(), team_items.begin() + r * G, team_items.begin() + (r + 1) * G);
    };
    for (long lo = 0, hi = R; lo < hi;) {
      round(lo++);
      if (lo < hi) round(--hi);
    }
    mixed.insert(mixed.end(), team_items.begin() + R * G, team_items.end());
    team_items.swap(mixed);
  }
  for (const RagItem& it : cta_items) {
    if (it.kind == kBig) plan->has_big = true;
    if (it.kind == kSingle) plan->max_single_rows = std::max(plan->max_single_rows, it.rows);
  }
  plan->items = std::move(cta_items);
  plan->items.insert(plan->items.end(), team_items.begin(), team_items.end());
  *plan_out = plan;
  return TRIDI_SUCCESS;
}
}  // namespace
}  // namespace tridi

extern "C" {

size_t tridi_ragged_plan_device_bytes(const void* plan) {
  return plan ? static_cast<const RaggedPlan*>(plan)->device_bytes() : 0;
}

long tridi_ragged_plan_total_rows(const void* plan) {
  return plan ? static_cast<const RaggedPlan*>(plan)->total_rows : 0;
}

int tridi_ragged_plan_num_systems(const void* plan) {
  return plan ? static_cast<const RaggedPlan*>(plan)->num_systems : 0;
}

int tridi_ragged_plan_items(const void* plan) {
  return plan ? (int)static_cast<const RaggedPlan*>(plan)->items.size() : 0;
}

// Copies the plan's item table into dev_buf (device memory of at least
// tridi_ragged_plan_device_bytes bytes), asynchronously on stream.
tridi_status tridi_ragged_plan_upload(const void* plan_, void* dev_buf, size_t bytes, tridi_stream_t stream) {
  using namespace tridi;
  const auto* plan = static_cast<const RaggedPlan*>(plan_);
  if (!plan || !dev_buf || bytes < plan->device_bytes()) return TRIDI_ERROR_INVALID_VALUE;
  char* d = static_cast<char*>(dev_buf);
  cudaStream_t st = as_stream(stream);
  cudaError_t e;
  if ((e = cudaMemsetAsync(d, 0, 64, st)) != cudaSuccess) return cuda_status(e);
  if ((e = cudaMemcpyAsync(d + 64, plan->items.data(), plan->items.size() * sizeof(RagItem),
                           cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_status(e);
  if ((e = cudaMemcpyAsync(d + 64 + plan->items.size() * sizeof(RagItem), plan->sys.data(),
                           plan->sys.size() * sizeof(RagSys), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_status(e);
  // the host vectors must stay alive until the copy ran: synchronise here,
  // plans are built once and reused.
  return cuda_status(cudaStreamSynchronize(st));
}

// Same as tridi_ragged_plan_upload without the final synchronisation: the
// caller keeps the plan alive until the copies on `stream` have run.
tridi_status tridi_ragged_plan_upload_async(const void* plan_, void* dev_buf, size_t bytes, tridi_stream_t stream) {
  using namespace tridi;
  const auto* plan = static_cast<const RaggedPlan*>(plan_);
  if (!plan || !dev_buf || bytes < plan->device_bytes()) return TRIDI_ERROR_INVALID_VALUE;
  char* d = static_cast<char*>(dev_buf);
  cudaStream_t st = as_stream(stream);
  cudaError_t e;
  if ((e = cudaMemsetAsync(d, 0, 64, st)) != cudaSuccess) return cuda_status(e);
  if ((e = cudaMemcpyAsync(d + 64, plan->items.data(), plan->items.size() * sizeof(RagItem),
                           cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_status(e);
  if ((e = cudaMemcpyAsync(d + 64 + plan->items.size() * sizeof(RagItem), plan->sys.data(),
                           plan->sys.size() * sizeof(RagSys), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_status(e);
  return TRIDI_SUCCESS;
}

tridi_status tridi_ragged_plan_destroy(void* plan) {
  delete static_cast<RaggedPlan*>(plan);
  return TRIDI_SUCCESS;
}

}  // extern "C"

namespace tridi {
namespace {

template <int MODE>
tridi_status ragged_launch(const RaggedPlan* plan, void* dev_plan, RagParams& p, cudaStream_t st) {
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  const size_t smem = rag_smem_bytes(MODE);
  if (smem > (size_t)dev->max_smem_optin) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  const auto kernel = plan->needs_big(ring_rows(MODE)) ? ragged_kernel<MODE, true> : ragged_kernel<MODE, false>;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return cuda_status(e);
  char* dp = static_cast<char*>(dev_plan);
  p.items = reinterpret_cast<const RagItem*>(dp + 64);
  p.sys = reinterpret_cast<const RagSys*>(dp + 64 + plan->items.size() * sizeof(RagItem));
  p.nitems = (int)plan->items.size();
  p.status = dev->status;
  int grid = dev->sm_count;
  if (grid > p.nitems) grid = p.nitems;
  kernel<<<grid, kRagThreads + 32, smem, st>>>(p);
  return cuda_status(cudaGetLastError());
}

long pad4(long v) { return (v + 3) & ~3L; }
long a64(long v) { return (v + 63) & ~63L; }

}  // namespace
}  // namespace tridi

extern "C" {

namespace tridi {
namespace {
__global__ void df_to_double_kernel(const float* hi, const float* lo, double* out, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = df_to_double(hi[i], lo[i]);
}
}  // namespace
}  // namespace tridi

// Self-check of the double-float -> FP64 assembly used by the refinement's
// output (device arrays of n elements).
tridi_status tridi_selfcheck_df_to_double(const float* hi, const float* lo, double* out, long n,
                                          tridi_stream_t stream) {
  if (!hi || !lo || !out || n < 0) return TRIDI_ERROR_INVALID_VALUE;
  if (n == 0) return TRIDI_SUCCESS;
  tridi::df_to_double_kernel<<<(unsigned)((n + 255) / 256), 256, 0, tridi::as_stream(stream)>>>(hi, lo, out, n);
  return tridi::cuda_status(cudaGetLastError());
}

// Solves every system of the plan.  a..d, x: concatenated rows (device,
// 16-byte aligned, at least round_up(total_rows, 4) elements).  dev_plan: the
// uploaded plan.  Stream-ordered and free of host synchronisation, so the
// call can be captured in a CUDA graph and replayed.
tridi_status tridi_ragged_solve_f32(const float* a, const float* b, const float* c, const float* d, float* x,
                                    const void* plan_, void* dev_plan, tridi_stream_t stream) {
  using namespace tridi;
  const auto* plan = static_cast<const RaggedPlan*>(plan_);
  if (!a || !b || !c || !d || !x || !plan || !dev_plan) return TRIDI_ERROR_INVALID_VALUE;
  if (!aligned16(a) || !aligned16(b) || !aligned16(c) || !aligned16(d)) return TRIDI_ERROR_MISALIGNED;
  RagParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  return ragged_launch<kPlain>(plan, dev_plan, p, as_stream(stream));
}

// Workspace of tridi_ragged_refine_f32: x (two words) and r of systems too
// large for the shared-memory ring, per row of the batch.
size_t tridi_ragged_refine_workspace_bytes(long total_rows, long num_systems) {
  (void)num_systems;
  return (size_t)tridi::a64(tridi::pad4(total_rows)) * 12 + 256;
}

// Fused refinement of every system of the plan (see the file comment):
// FP32 solves in shared memory, residual and accumulation in extended
// precision (TRIDI_TUNE_RESIDUAL: double-float by default, native FP64 on
// request), `sweeps` corrections, x written once in FP64.  *dev_rel (device
// double) receives max over systems of ||d - T x||_2 / ||d||_2.  offsets_dev
// is accepted for interface stability and not needed.  Stream-ordered, no
// host synchronisation (capturable in a CUDA graph).
tridi_status tridi_ragged_refine_f32(const float* a, const float* b, const float* c, const float* d, double* x,
                                     const void* plan_, void* dev_plan, const long* offsets_dev, int sweeps,
                                     void* ws, size_t ws_bytes, double* dev_rel, tridi_stream_t stream) {
  using namespace tridi;
  (void)offsets_dev;
  const auto* plan = static_cast<const RaggedPlan*>(plan_);
  if (!a || !b || !c || !d || !x || !plan || !dev_plan || !ws || !dev_rel || sweeps < 0)
    return TRIDI_ERROR_INVALID_VALUE;
  if (!aligned16(a) || !aligned16(b) || !aligned16(c) || !aligned16(d)) return TRIDI_ERROR_MISALIGNED;
  const long total = plan->total_rows;
  if (ws_bytes < tridi_ragged_refine_workspace_bytes(total, plan->num_systems))
    return TRIDI_ERROR_WORKSPACE_TOO_SMALL;
  const long rows = a64(pad4(total));
  cudaStream_t st = as_stream(stream);
  cudaError_t ce;
  if ((ce = cudaMemsetAsync(dev_rel, 0, sizeof(double), st)) != cudaSuccess) return cuda_status(ce);
  RagParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x64 = x;
  p.wxh = static_cast<float*>(ws);
  p.wxl = p.wxh + rows;
  p.wr = p.wxl + rows;
  p.rel = reinterpret_cast<unsigned long long*>(dev_rel);
  p.sweeps = sweeps;
  const int res = tunable(TRIDI_TUNE_RESIDUAL);
  if (res != 0 && res != TRIDI_RESIDUAL_DF && res != TRIDI_RESIDUAL_FP64) return TRIDI_ERROR_INVALID_VALUE;
  const bool fp64 = res == TRIDI_RESIDUAL_FP64;
  if (sweeps == 1)  // x0 and its correction in the ring's b and d words
    return fp64 ? ragged_launch<kRefine1FP64>(plan, dev_plan, p, st) : ragged_launch<kRefine1DF>(plan, dev_plan, p, st);
  return fp64 ? ragged_launch<kRefineFP64>(plan, dev_plan, p, st) : ragged_launch<kRefineDF>(plan, dev_plan, p, st);
}

}  // extern "C"

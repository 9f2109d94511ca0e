// Ragged batches: systems of different sizes, concatenated (system s owns rows
// [off[s], off[s+1]) of a, b, c, d, x), solved by ONE persistent launch.
// No counterpart in the reference (its launchers take one size per call).
//
// Work queue.  The host plan (tridi_ragged_plan_*) sorts the systems into
// size buckets and cuts them into work items, largest first:
//   MULTI  up to 15 systems of <= 480 rows: one warp per system
//   MULTI4 up to 3 systems of 481 .. 2400 rows: 160 threads (own named
//          barrier) per system, three systems at once
//   SINGLE one system of 2401 .. ~6140 rows: the whole CTA
//   DOUBLE one system of up to 12280 rows: the whole CTA, both stage buffers
//   BIG    one system of up to 24480 rows, read from global memory (no
//          staging): every thread owns three chunks of up to 17 rows; pass 1
//          eliminates them and exports their interfaces, the 1440
//          separators are solved by PCR in shared memory, pass 2 eliminates
//          again (rows now in L2) and substitutes back
// One CTA per SM (480 consumer threads + a producer warp).  Items are sorted
// largest first and CTA b takes items b, b + grid, b + 2 grid, ... (so every
// CTA gets the same mix of sizes, and no claim has to wait on an atomic).
// Its producer stages each item into one of two shared-memory buffers with
// cp.async.bulk (each system's 16-byte-aligned row range, per array) while
// the consumers solve the previous one, and publishes the item through the
// stage's mbarrier; a DOUBLE waits for both buffers.
// Arithmetic: the partition solver of partition.cuh, per warp (MULTI), per
// group of 160 threads (MULTI4) or per CTA (SINGLE / DOUBLE), with the chunk
// elimination done in place in the stage buffer (no register arrays, so no
// bound on rows per thread) and the separators solved by PCR in shuffles
// (warp) or shared memory (group, CTA).
// The arrays must hold at least round_up(total_rows, 4) elements and be
// 16-byte aligned (the bulk copies read whole 16-byte groups).
#include <algorithm>
#include <cstring>
#include <vector>

#include "partition.cuh"
#include "runtime.h"

namespace tridi {

constexpr int kRagThreads = 480;       // consumer threads per CTA (15 warps; + 1 producer warp = 16 warps,
                                       // 4 per SM sub-partition, so up to 128 registers per thread)
constexpr int kRagWarps = kRagThreads / 32;
constexpr int kStageRows = 6144;       // rows per stage buffer (per array)
constexpr int kWarpMaxRows = 480;      // MULTI systems: up to 15 rows per lane
constexpr int kMaxItemSystems = kRagWarps;       // 15
constexpr int kMaxSystemRows = 2 * kStageRows - 8;  // 12280: largest staged system (a DOUBLE item)
constexpr int kBigChunks = 3;                      // chunks per thread for BIG systems
constexpr int kBigSepRows = kBigChunks * kRagThreads;      // chunks (separators) of a BIG system
constexpr int kMaxBigRows = 17 * kBigSepRows;              // 24480

enum ItemKind : int { kMulti = 0, kSingle = 1, kDouble = 2, kNop = 3, kCont = 4, kEnd = 5, kBig = 6, kMulti4 = 7 };
constexpr int kGroup4Threads = 160;                    // MULTI4: threads per system (5 warps)
constexpr int kGroup4MaxRows = 2400;                   // MULTI4 systems: up to 15 rows per thread

struct RagItem {
  int kind;
  int count;        // systems in the item
  int first;        // index into the plan's system list
  int rows;         // padded rows the item occupies in the stage (per array)
};

// Plan buffer on the device: [counter (16 B)] [items] [system list].
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
  float* x;
  const RagItem* items;
  const RagSys* sys;
  int nitems;
  unsigned* counter;
  unsigned* status;
};

struct RagStage {  // per-stage descriptor published by the producer
  int item;        // index into items, or -1 for NOP / CONT / END markers
  int kind;
  int base[kMaxItemSystems];  // row of each system's first row inside the stage
};

__device__ __forceinline__ int odd_ceil_dev(int v) { return (v & 1) ? v : v + 1; }

// Named barrier over `count` threads with a runtime id (1 = all consumers,
// 2.. = MULTI4 groups).
__device__ __forceinline__ void group_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// One system of n rows (shared-memory arrays sa..sd, overwritten) solved by a
// group of gt threads (thread gtid of the group; gt == 32: one warp, else a
// named barrier `bar` over the group): chunk elimination in place, the gt
// separators solved by PCR (warp shuffles, or shared memory R: 4*gt floats,
// X: gt, F0: 3*(gt/32)), back substitution; x written to global memory.
__device__ __forceinline__ void group_solve(int n, int gt, int bar, int gtid, float* sa, const float* sb, float* sc,
                                            float* sd, float* R, float* X, float* F0, float* xg) {
  const int lane = gtid & 31, gw = gtid >> 5;
  const int kk = odd_ceil_dev((n + gt - 1) / gt);
  const int r0 = gtid * kk;
  int kr = n - r0;
  kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
  ChunkSummary<float> cs;
  chunk_eliminate_smem<float>(cs, kr, gtid == 0, r0 + kr == n && kr > 0, sa + r0, sb + r0, sc + r0, sd + r0);
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
    const Row<float> id{0.f, 1.f, 0.f, 0.f};
    for (int dl = 1; dl < gt; dl *= 2) {
      R[gtid] = sr.a; R[gt + gtid] = sr.b; R[2 * gt + gtid] = sr.c; R[3 * gt + gtid] = sr.d;
      group_sync(bar, gt);
      const Row<float> L = gtid >= dl ? Row<float>{R[gtid - dl], R[gt + gtid - dl], R[2 * gt + gtid - dl],
                                                   R[3 * gt + gtid - dl]}
                                      : id;
      const Row<float> Rr = gtid + dl < gt ? Row<float>{R[gtid + dl], R[gt + gtid + dl], R[2 * gt + gtid + dl],
                                                        R[3 * gt + gtid + dl]}
                                           : id;
      sr = reduce_row(sr, L, Rr);
      group_sync(bar, gt);
    }
    sj = tdiv(sr.d, sr.b);
    X[gtid] = sj;
    group_sync(bar, gt);
    sl = gtid > 0 ? X[gtid - 1] : 0.f;
  }
  chunk_back_smem<float>(kr, sj, sl, sa + r0, sc + r0, sd + r0, xg + r0);
  if (gt != 32) group_sync(bar, gt);  // F0 / R / X reused by the next item
}

// A BIG system (rows read straight from global memory): kBigSepRows chunks,
// kBigChunks per consumer thread; their separators solved by PCR across the
// consumers in shared memory, then every chunk eliminated again and
// substituted back.
__device__ __forceinline__ void solve_big(RagSys sy, const float* __restrict__ a, const float* __restrict__ b,
                                       const float* __restrict__ c, const float* __restrict__ d, float* x, int tid,
                                       float* Rsh, float* Xsh, float* Fb) {
  const int n = sy.n;
  constexpr int KC = 17;
  constexpr int NS = kBigSepRows;  // chunks (= separators) of the system
  const int kk = odd_ceil_dev((n + NS - 1) / NS);
  const float* ga = a + sy.off;
  const float* gb = b + sy.off;
  const float* gc = c + sy.off;
  const float* gd = d + sy.off;
  // pass 1: eliminate every chunk; export its first-row coefficients (Fb)
  // and the part of its separator row that needs no neighbour (Rsh)
#pragma unroll 1
  for (int q = 0; q < kBigChunks; ++q) {
    const int j = q * kRagThreads + tid;
    const int r0 = j * kk;
    int kr = n - r0;
    kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
    Chunk<float, KC> ch;
    chunk_eliminate<float, KC>(ch, kr, j == 0, r0 + kr == n && kr > 0, ga + r0, gb + r0, gc + r0,
                                     gd + r0);
    Fb[3 * j + 0] = ch.fD; Fb[3 * j + 1] = ch.fC; Fb[3 * j + 2] = ch.fA;
    const Row<float>& e = ch.sep;
    Rsh[j] = -e.a * ch.lA; Rsh[NS + j] = e.b - e.a * ch.lC; Rsh[2 * NS + j] = e.c;
    Rsh[3 * NS + j] = e.d - e.a * ch.lD;
  }
  consumer_sync(kRagThreads);
  // separator rows (the next chunk's first row folded in); PCR over all NS
  // of them, kBigChunks rows per thread
  Row<float> sr[kBigChunks];
#pragma unroll
  for (int q = 0; q < kBigChunks; ++q) {
    const int j = q * kRagThreads + tid;
    const float nD = j + 1 < NS ? Fb[3 * (j + 1) + 0] : 0.f;
    const float nC = j + 1 < NS ? Fb[3 * (j + 1) + 1] : 0.f;
    const float nA = j + 1 < NS ? Fb[3 * (j + 1) + 2] : 0.f;
    const float ec = Rsh[2 * NS + j];
    sr[q] = Row<float>{Rsh[j], Rsh[NS + j] - ec * nA, -ec * nC, Rsh[3 * NS + j] - ec * nD};
  }
  consumer_sync(kRagThreads);  // every partial row read before PCR overwrites Rsh
  const Row<float> id{0.f, 1.f, 0.f, 0.f};
  for (int dl = 1; dl < NS; dl *= 2) {
#pragma unroll
    for (int q = 0; q < kBigChunks; ++q) {
      const int j = q * kRagThreads + tid;
      Rsh[j] = sr[q].a; Rsh[NS + j] = sr[q].b; Rsh[2 * NS + j] = sr[q].c; Rsh[3 * NS + j] = sr[q].d;
    }
    consumer_sync(kRagThreads);
#pragma unroll
    for (int q = 0; q < kBigChunks; ++q) {
      const int j = q * kRagThreads + tid;
      const Row<float> L = j >= dl ? Row<float>{Rsh[j - dl], Rsh[NS + j - dl], Rsh[2 * NS + j - dl],
                                                Rsh[3 * NS + j - dl]}
                                   : id;
      const Row<float> R = j + dl < NS ? Row<float>{Rsh[j + dl], Rsh[NS + j + dl], Rsh[2 * NS + j + dl],
                                                    Rsh[3 * NS + j + dl]}
                                       : id;
      sr[q] = reduce_row(sr[q], L, R);
    }
    consumer_sync(kRagThreads);
  }
#pragma unroll
  for (int q = 0; q < kBigChunks; ++q) Xsh[q * kRagThreads + tid] = tdiv(sr[q].d, sr[q].b);
  consumer_sync(kRagThreads);
  // pass 2: eliminate again and substitute back
#pragma unroll 1
  for (int q = 0; q < kBigChunks; ++q) {
    const int j = q * kRagThreads + tid;
    const int r0 = j * kk;
    int kr = n - r0;
    kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
    Chunk<float, KC> ch;
    chunk_eliminate<float, KC>(ch, kr, j == 0, r0 + kr == n && kr > 0, ga + r0, gb + r0, gc + r0,
                                     gd + r0);
    chunk_back_store<float, KC>(ch, kr, Xsh[j], j > 0 ? Xsh[j - 1] : 0.f, x + sy.off + r0);
  }
  consumer_sync(kRagThreads);  // Fb / Xsh reused by the next item
}

__global__ void __launch_bounds__(kRagThreads + 32, 1) ragged_kernel(RagParams p) {
  static_assert((kRagThreads + 32) % 128 == 0, "16 warps: 4 per SM sub-partition");
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + 2;
  RagStage* desc = reinterpret_cast<RagStage*>(smem + 64);
  float* buf = reinterpret_cast<float*>(smem + 64 + 2 * sizeof(RagStage) + 64 - ((64 + 2 * sizeof(RagStage)) % 64));
  // buf layout: array q (a, b, c, d) occupies [q * 2 * kStageRows, (q+1) * 2 * kStageRows);
  // stage s is the half [s * kStageRows, (s+1) * kStageRows) of every array.
  float* Rsh = buf + 4 * 2 * kStageRows;  // group / CTA separators: 4 x kRagThreads
  float* Xsh = Rsh + 4 * kRagThreads;     // their solution
  float* F0 = Xsh + kRagThreads;          // lane-0 first-row coefficients of each warp (3 x kRagWarps)
  // A BIG item stages nothing: its separators (4 x kBigSepRows) use the a-half
  // of its stage, their solution and the chunks' first-row coefficients
  // (kBigSepRows + 3 x kBigSepRows) the b-half.
  static_assert(4 * kBigSepRows <= kStageRows, "BIG scratch fits the halves of one stage");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kRagWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (tid >= kRagThreads) {  // ---------------- producer ----------------
    if (lane != 0) return;
    int k = 0;  // slot counter; slot k uses stage k & 1
    bool done = false;
    int next = blockIdx.x;
    while (!done) {
      int item = next < p.nitems ? next : -1;
      next += gridDim.x;
      const int kind = item >= 0 ? p.items[item].kind : (int)kEnd;
      if (kind == kDouble && (k & 1)) {  // a DOUBLE starts on stage 0: pad with a NOP
        if (k >= 2 && !mbar_wait(&empty[1], ((k >> 1) - 1) & 1, p.status)) break;
        desc[1].item = -1;
        desc[1].kind = kNop;
        mbar_arrive(&full[1]);
        ++k;
      }
      const int s = k & 1;
      if (k >= 2 && !mbar_wait(&empty[s], ((k >> 1) - 1) & 1, p.status)) break;
      // A DOUBLE (always on stage 0 here) also needs stage 1, last used at slot k-1.
      if (kind == kDouble && k >= 1 && !mbar_wait(&empty[1], ((k - 1) >> 1) & 1, p.status)) break;
      desc[s].item = item;
      desc[s].kind = kind;
      if (kind == kEnd) {
        mbar_arrive(&full[s]);
        done = true;
        break;
      }
      if (kind == kBig) {  // rows are read from global memory by the consumers
        mbar_arrive(&full[s]);
        ++k;
        continue;
      }
      const RagItem it = p.items[item];
      // Bytes of the whole item first: the single arrive carries the full
      // transaction count, so the phase cannot complete before every copy.
      uint32_t tx = 0;
      int cursor = s * kStageRows;
      for (int q = 0; q < it.count; ++q) {
        const RagSys sy = p.sys[it.first + q];
        const long lo = sy.off & ~3L, hi = (sy.off + sy.n + 3) & ~3L;
        desc[s].base[q] = cursor + (int)(sy.off - lo);
        tx += 4u * (uint32_t)((hi - lo) * 4);
        cursor += (int)(hi - lo);
      }
      mbar_arrive_expect_tx(&full[s], tx);
      cursor = s * kStageRows;
      for (int q = 0; q < it.count; ++q) {
        const RagSys sy = p.sys[it.first + q];
        const long lo = sy.off & ~3L, hi = (sy.off + sy.n + 3) & ~3L;
        const uint32_t bytes = (uint32_t)((hi - lo) * 4);
        bulk_g2s(buf + 0 * 2 * kStageRows + cursor, p.a + lo, bytes, &full[s]);
        bulk_g2s(buf + 1 * 2 * kStageRows + cursor, p.b + lo, bytes, &full[s]);
        bulk_g2s(buf + 2 * 2 * kStageRows + cursor, p.c + lo, bytes, &full[s]);
        bulk_g2s(buf + 3 * 2 * kStageRows + cursor, p.d + lo, bytes, &full[s]);
        cursor += (int)(hi - lo);
      }
      ++k;
      if (kind == kDouble) {  // the second buffer belongs to this item: publish a continuation
        desc[1].item = -1;
        desc[1].kind = kCont;
        mbar_arrive(&full[1]);
        ++k;
      }
    }
    return;
  }

  // ---------------- consumers ----------------
  float* A = buf;  // the consumers overwrite a, c, d of a staged item in place
  const float* B = buf + 2 * kStageRows;
  float* C = buf + 4 * kStageRows;
  float* D = buf + 6 * kStageRows;
  for (int k = 0;; ++k) {
    const int s = k & 1;
    const bool ok = consumer_sync_and(kRagThreads, mbar_wait(&full[s], (k >> 1) & 1, p.status));
    if (!ok) break;
    const int kind = desc[s].kind;
    if (kind == kEnd) break;
    if (kind == kMulti) {
      const RagItem it = p.items[desc[s].item];
      if (warp < it.count) {
        const RagSys sy = p.sys[it.first + warp];
        const int base = desc[s].base[warp];
        group_solve(sy.n, 32, 0, lane, A + base, B + base, C + base, D + base, nullptr, nullptr, nullptr,
                    p.x + sy.off);
      }
    } else if (kind == kMulti4) {
      const RagItem it = p.items[desc[s].item];
      const int g = tid / kGroup4Threads;
      if (g < it.count) {
        const RagSys sy = p.sys[it.first + g];
        const int base = desc[s].base[g];
        group_solve(sy.n, kGroup4Threads, 2 + g, tid - g * kGroup4Threads, A + base, B + base, C + base, D + base,
                    Rsh + g * 4 * kGroup4Threads, Xsh + g * kGroup4Threads, F0 + g * 3 * (kGroup4Threads / 32),
                    p.x + sy.off);
      }
    } else if (kind == kSingle || kind == kDouble) {
      const RagItem it = p.items[desc[s].item];
      const RagSys sy = p.sys[it.first];
      const int base = desc[s].base[0];
      group_solve(sy.n, kRagThreads, 1, tid, A + base, B + base, C + base, D + base, Rsh, Xsh, F0, p.x + sy.off);
    } else if (kind == kBig) {
      const RagItem it = p.items[desc[s].item];
      float* bR = buf + s * kStageRows;
      float* bX = buf + 2 * kStageRows + s * kStageRows;
      solve_big(p.sys[it.first], p.a, p.b, p.c, p.d, p.x, tid, bR, bX, bX + kBigSepRows);
    }
    release_stage(&empty[s]);
  }
}

// ---------------------------------------------------------------------------
// Host plan.
struct RaggedPlan {
  std::vector<RagItem> items;
  std::vector<RagSys> sys;
  long total_rows = 0;
  int num_systems = 0;
  size_t device_bytes() const {
    return 64 + items.size() * sizeof(RagItem) + sys.size() * sizeof(RagSys);
  }
};

namespace {
size_t rag_smem_bytes() {
  size_t head = 64 + 2 * sizeof(RagStage);
  head += 64 - head % 64;
  return head + (size_t)(4 * 2 * kStageRows + 5 * kRagThreads + 3 * kRagWarps) * sizeof(float);
}
long padded_rows(long off, int n) { return ((off + n + 3) & ~3L) - (off & ~3L); }
}  // namespace

}  // namespace tridi

using tridi::RaggedPlan;

extern "C" {

tridi_status tridi_ragged_plan_create(const long* offsets, int num_systems, void** plan_out) {
  using namespace tridi;
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
  int i = 0;
  while (i < num_systems) {
    const RagSys& sy = plan->sys[i];
    const long pr = padded_rows(sy.off, sy.n);
    if (sy.n > kMaxSystemRows || pr > 2 * kStageRows) {
      plan->items.push_back(RagItem{(int)kBig, 1, i, 0});
      ++i;
      continue;
    }
    if (sy.n > kGroup4MaxRows) {
      RagItem it{pr > kStageRows ? (int)kDouble : (int)kSingle, 1, i, (int)pr};
      plan->items.push_back(it);
      ++i;
      continue;
    }
    if (sy.n > kWarpMaxRows) {
      RagItem it{(int)kMulti4, 0, i, 0};
      while (i < num_systems && it.count < kRagThreads / kGroup4Threads) {
        const RagSys& t = plan->sys[i];
        const long tr = padded_rows(t.off, t.n);
        if (t.n > kGroup4MaxRows || t.n <= kWarpMaxRows || it.rows + tr > kStageRows) break;
        it.rows += (int)tr;
        ++it.count;
        ++i;
      }
      plan->items.push_back(it);
      continue;
    }
    RagItem it{(int)kMulti, 0, i, 0};
    while (i < num_systems && it.count < kMaxItemSystems) {
      const RagSys& t = plan->sys[i];
      const long tr = padded_rows(t.off, t.n);
      if (t.n > kWarpMaxRows || it.rows + tr > kStageRows) break;
      it.rows += (int)tr;
      ++it.count;
      ++i;
    }
    plan->items.push_back(it);
  }
  *plan_out = plan;
  return TRIDI_SUCCESS;
}

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

// Solves every system of the plan.  a..d, x: concatenated rows (device,
// 16-byte aligned, at least round_up(total_rows, 4) elements).  dev_plan: the
// uploaded plan.  Stream-ordered; resets the work counter itself (a memset),
// so the call can be captured in a CUDA graph and replayed.
tridi_status tridi_ragged_solve_f32(const float* a, const float* b, const float* c, const float* d, float* x,
                                    const void* plan_, void* dev_plan, tridi_stream_t stream) {
  using namespace tridi;
  const auto* plan = static_cast<const RaggedPlan*>(plan_);
  if (!a || !b || !c || !d || !x || !plan || !dev_plan) return TRIDI_ERROR_INVALID_VALUE;
  if (!aligned16(a) || !aligned16(b) || !aligned16(c) || !aligned16(d)) return TRIDI_ERROR_MISALIGNED;
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  const size_t smem = rag_smem_bytes();
  if (smem > (size_t)dev->max_smem_optin) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  cudaStream_t st = as_stream(stream);
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(ragged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
      cudaSuccess)
    return cuda_status(e);
  char* dp = static_cast<char*>(dev_plan);
  if ((e = cudaMemsetAsync(dp, 0, 64, st)) != cudaSuccess) return cuda_status(e);
  RagParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.items = reinterpret_cast<const RagItem*>(dp + 64);
  p.sys = reinterpret_cast<const RagSys*>(dp + 64 + plan->items.size() * sizeof(RagItem));
  p.nitems = (int)plan->items.size();
  p.counter = reinterpret_cast<unsigned*>(dp);
  p.status = dev->status;
  int grid = dev->sm_count;
  if (grid > p.nitems) grid = p.nitems;
  ragged_kernel<<<grid, kRagThreads + 32, smem, st>>>(p);
  return cuda_status(cudaGetLastError());
}

}  // extern "C"

// Ragged batches: systems of different sizes, concatenated (system s owns rows
// [off[s], off[s+1]) of a, b, c, d, x), solved by ONE persistent launch.
// No counterpart in the reference (its launchers take one size per call).
//
// Work queue.  The host plan (tridi_ragged_plan_*) sorts the systems into
// size buckets and cuts them into work items, largest first:
//   MULTI  up to 16 systems of <= 480 rows: one warp per system
//   SINGLE one system of 481 .. kStageRows-3 rows: the whole CTA
//   DOUBLE one system of up to 8704 rows: the whole CTA, both stage buffers
//   BIG    one system of up to 17408 rows, read from global memory (no
//          staging): every thread owns two chunks; pass 1 eliminates them
//          and exports their interfaces, the 1024 separators are solved by
//          PCR in shared memory, pass 2 eliminates again (rows now in L2)
//          and substitutes back
// One CTA per SM (512 consumer threads + a producer warp).  The producer
// claims the next item with an atomicAdd on a counter in the plan buffer,
// stages it into one of two shared-memory buffers with cp.async.bulk (each
// system's 16-byte-aligned row range, per array), and publishes the item
// index through the stage's mbarrier.  Items therefore flow to whichever SM
// is free (dynamic load balance); a DOUBLE waits for both buffers.
// Arithmetic: the partition solver of partition.cuh, per warp (MULTI) or per
// CTA with a shared-memory PCR on the CTA's separators (SINGLE / DOUBLE).
// The arrays must hold at least round_up(total_rows, 4) elements and be
// 16-byte aligned (the bulk copies read whole 16-byte groups).
#include <algorithm>
#include <cstring>
#include <vector>

#include "partition.cuh"
#include "runtime.h"

namespace tridi {

constexpr int kRagThreads = 512;       // consumer threads per CTA
constexpr int kRagWarps = kRagThreads / 32;
constexpr int kStageRows = 6144;       // rows per stage buffer (per array)
constexpr int kWarpMaxRows = 480;      // MULTI systems: 32 lanes x 15 rows
constexpr int kMaxItemSystems = 16;
constexpr int kMaxSystemRows = 17 * kRagThreads;  // 8704: largest staged system
constexpr int kBigChunks = 2;                      // chunks per thread for BIG systems
constexpr int kMaxBigRows = kBigChunks * 17 * kRagThreads;  // 17408

enum ItemKind : int { kMulti = 0, kSingle = 1, kDouble = 2, kNop = 3, kCont = 4, kEnd = 5, kBig = 6 };

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

__global__ void __launch_bounds__(kRagThreads + 32, 1) ragged_kernel(RagParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + 2;
  RagStage* desc = reinterpret_cast<RagStage*>(smem + 64);
  float* buf = reinterpret_cast<float*>(smem + 64 + 2 * sizeof(RagStage) + 64 - ((64 + 2 * sizeof(RagStage)) % 64));
  // buf layout: array q (a, b, c, d) occupies [q * 2 * kStageRows, (q+1) * 2 * kStageRows);
  // stage s is the half [s * kStageRows, (s+1) * kStageRows) of every array.
  constexpr int kSepRows = kBigChunks * kRagThreads;
  float* Rsh = buf + 4 * 2 * kStageRows;  // CTA-mode separators: 4 x kSepRows
  float* Xsh = Rsh + 4 * kSepRows;        // their solution
  float* F0 = Xsh + kSepRows;             // lane-0 first-row coefficients of each warp (3 x kRagWarps)
  float* Fb = F0 + 3 * kRagWarps;         // BIG: first-row coefficients of every chunk (3 x kSepRows)
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
    while (!done) {
      int item = (int)atomicAdd(p.counter, 1u);
      if (item >= p.nitems) item = -1;
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
  const float* A = buf;
  const float* B = buf + 2 * kStageRows;
  const float* C = buf + 4 * kStageRows;
  const float* D = buf + 6 * kStageRows;
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
        const int n = sy.n;
        const int kk = odd_ceil_dev((n + 31) / 32);
        float xr[15];
        const int kl = warp_partition_solve<float, 15>(n, kk, A + base, B + base, C + base, D + base, xr);
        float* dst = p.x + sy.off + lane * kk;
#pragma unroll
        for (int i = 0; i < 15; ++i)
          if (i < kl) dst[i] = xr[i];
      }
    } else if (kind == kSingle || kind == kDouble) {
      const RagItem it = p.items[desc[s].item];
      const RagSys sy = p.sys[it.first];
      const int base = desc[s].base[0];
      const int n = sy.n;
      const int kk = odd_ceil_dev((n + kRagThreads - 1) / kRagThreads);
      const int r0 = tid * kk;
      int kr = n - r0;
      kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
      constexpr int KC = 17;  // rows per thread: systems of up to 17 * 512 = 8704 rows
      Chunk<float, KC> ch;
      chunk_eliminate<float, KC>(ch, kr, tid == 0, r0 + kr == n && kr > 0, A + base + r0, B + base + r0,
                                 C + base + r0, D + base + r0);
      if (lane == 0) {
        F0[warp * 3 + 0] = ch.fD; F0[warp * 3 + 1] = ch.fC; F0[warp * 3 + 2] = ch.fA;
      }
      consumer_sync(kRagThreads);
      float nD = __shfl_down_sync(kFull, ch.fD, 1);
      float nC = __shfl_down_sync(kFull, ch.fC, 1);
      float nA = __shfl_down_sync(kFull, ch.fA, 1);
      if (lane == 31 && warp + 1 < kRagWarps) {
        nD = F0[(warp + 1) * 3 + 0]; nC = F0[(warp + 1) * 3 + 1]; nA = F0[(warp + 1) * 3 + 2];
      }
      Row<float> sr = separator_row<float, KC>(ch, nD, nC, nA);
      const Row<float> id{0.f, 1.f, 0.f, 0.f};
      for (int dl = 1; dl < kRagThreads; dl *= 2) {
        Rsh[tid] = sr.a; Rsh[kRagThreads + tid] = sr.b; Rsh[2 * kRagThreads + tid] = sr.c;
        Rsh[3 * kRagThreads + tid] = sr.d;
        consumer_sync(kRagThreads);
        const Row<float> L = tid >= dl ? Row<float>{Rsh[tid - dl], Rsh[kRagThreads + tid - dl],
                                                    Rsh[2 * kRagThreads + tid - dl], Rsh[3 * kRagThreads + tid - dl]}
                                       : id;
        const Row<float> R = tid + dl < kRagThreads
                                 ? Row<float>{Rsh[tid + dl], Rsh[kRagThreads + tid + dl],
                                              Rsh[2 * kRagThreads + tid + dl], Rsh[3 * kRagThreads + tid + dl]}
                                 : id;
        sr = reduce_row(sr, L, R);
        consumer_sync(kRagThreads);
      }
      Xsh[tid] = tdiv(sr.d, sr.b);
      consumer_sync(kRagThreads);
      const float sj = Xsh[tid];
      const float sl = tid > 0 ? Xsh[tid - 1] : 0.f;
      float xr[KC];
      chunk_back<float, KC>(ch, kr, sj, sl, xr);
      float* dst = p.x + sy.off + r0;
#pragma unroll
      for (int i = 0; i < KC; ++i)
        if (i < kr) dst[i] = xr[i];
      consumer_sync(kRagThreads);  // F0 / Xsh reused by the next item
    } else if (kind == kBig) {
      const RagItem it = p.items[desc[s].item];
      const RagSys sy = p.sys[it.first];
      const int n = sy.n;
      constexpr int KC = 17;
      constexpr int NS = kSepRows;  // chunks (= separators) of the system
      const int kk = odd_ceil_dev((n + NS - 1) / NS);
      const float* ga = p.a + sy.off;
      const float* gb = p.b + sy.off;
      const float* gc = p.c + sy.off;
      const float* gd = p.d + sy.off;
      // pass 1: eliminate both chunks, export first-row coefficients to shared
      // memory and keep the last-row coefficients and separator rows
      Row<float> sep[kBigChunks];
      float lD[kBigChunks], lC[kBigChunks], lA[kBigChunks];
#pragma unroll
      for (int q = 0; q < kBigChunks; ++q) {
        const int j = q * kRagThreads + tid;
        const int r0 = j * kk;
        int kr = n - r0;
        kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
        Chunk<float, KC> ch;
        chunk_eliminate<float, KC>(ch, kr, j == 0, r0 + kr == n && kr > 0, ga + r0, gb + r0, gc + r0,
                                         gd + r0);
        Fb[3 * j + 0] = ch.fD; Fb[3 * j + 1] = ch.fC; Fb[3 * j + 2] = ch.fA;
        sep[q] = ch.sep; lD[q] = ch.lD; lC[q] = ch.lC; lA[q] = ch.lA;
      }
      consumer_sync(kRagThreads);
      // separator rows; PCR over all NS of them, kBigChunks rows per thread
      Row<float> sr[kBigChunks];
#pragma unroll
      for (int q = 0; q < kBigChunks; ++q) {
        const int j = q * kRagThreads + tid;
        const float nD = j + 1 < NS ? Fb[3 * (j + 1) + 0] : 0.f;
        const float nC = j + 1 < NS ? Fb[3 * (j + 1) + 1] : 0.f;
        const float nA = j + 1 < NS ? Fb[3 * (j + 1) + 2] : 0.f;
        const Row<float>& e = sep[q];
        sr[q] = Row<float>{-e.a * lA[q], e.b - e.a * lC[q] - e.c * nA, -e.c * nC, e.d - e.a * lD[q] - e.c * nD};
      }
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
#pragma unroll
      for (int q = 0; q < kBigChunks; ++q) {
        const int j = q * kRagThreads + tid;
        const int r0 = j * kk;
        int kr = n - r0;
        kr = kr < 0 ? 0 : (kr > kk ? kk : kr);
        Chunk<float, KC> ch;
        chunk_eliminate<float, KC>(ch, kr, j == 0, r0 + kr == n && kr > 0, ga + r0, gb + r0, gc + r0,
                                         gd + r0);
        float xr[KC];
        chunk_back<float, KC>(ch, kr, Xsh[j], j > 0 ? Xsh[j - 1] : 0.f, xr);
        float* dst = p.x + sy.off + r0;
#pragma unroll
        for (int i = 0; i < KC; ++i)
          if (i < kr) dst[i] = xr[i];
      }
      consumer_sync(kRagThreads);  // Fb / Xsh reused by the next item
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
  return head + (size_t)(4 * 2 * kStageRows + 5 * kBigChunks * kRagThreads + 3 * kRagWarps +
                         3 * kBigChunks * kRagThreads) * sizeof(float);
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
    if (sy.n > kWarpMaxRows) {
      RagItem it{pr > kStageRows ? (int)kDouble : (int)kSingle, 1, i, (int)pr};
      plan->items.push_back(it);
      ++i;
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

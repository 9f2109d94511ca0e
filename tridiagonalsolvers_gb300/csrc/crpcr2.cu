// CR-PCR with the switch at half the system ("crpcr" with restSystemSize =
// n/2, crpcr_kernel.cu:1-148, crpcr_app.cu:5) for FP32 systems of 1024
// unknowns, in registers: one CR level, PCR on the 512-row intermediate
// system, the CR back substitution.
//
// A warp holds one system, 32 contiguous rows a lane (the 1024-row tile of
// pcr_twophase.cuh).  The CR level eliminates the even rows from the odd ones
// inside the lane (the last odd row's right neighbour is the next lane's
// first row, one shuffle): lane t keeps the intermediate rows 16t .. 16t+15
// (original rows 32t + 2j + 1) as normalised 3-word rows -- exactly the
// 512-row layout of the two-phase PCR (16 rows a lane, one system a warp), so
// its phase A, transpose, phase B and closing 2x2 systems run unchanged and
// leave x of intermediate row t + 32s in lane t.  Those 512 values go through
// the warp's scratch once (padded so the lane-contiguous reads hit distinct
// banks), each lane forms its 16 even rows' x from its own coefficients, and
// writes its 32 unknowns with 16-byte stores.
#include "hybrid.cuh"
#include "pcr_twophase.cuh"
#include "runtime.h"

namespace tridi {

namespace {

using namespace pcr2;

constexpr int kN = 1024;
constexpr int kR = 32;          // original rows a lane
constexpr int kRR = 16;         // intermediate rows a lane
constexpr int kLPS = 32;        // lanes per system
constexpr int kTF = kN;         // values of one array in a warp tile (one system)
constexpr int kWarps = 2;       // warps per CTA
constexpr int kScratch = 512 + 32;  // one word array of the 512-row transpose, then x of the 512 rows (padded)
constexpr size_t kSmem = 128 + (size_t)kWarps * kScratch * sizeof(float) + 1024 + (size_t)kWarps * 4 * kTF * 4;

constexpr size_t kSmem256 = 128 + (size_t)kWarps * 3 * (256 + 32) * sizeof(float) + 1024 + (size_t)kWarps * 4 * kTF * 4;

__device__ __forceinline__ int xr_index(int r) { return r + (r >> 4); }  // one pad word per 16

__global__ void __launch_bounds__(kWarps * 32, 3)
    crpcr512_kernel(HybridParams p, const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                    const __grid_constant__ CUtensorMap mc, const __grid_constant__ CUtensorMap md) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + warp;
  float* sw = reinterpret_cast<float*>(smem + 128) + (size_t)warp * kScratch;
  const uint32_t base = smem_addr(smem);
  const uint32_t ring = (base + 128 + kWarps * kScratch * (uint32_t)sizeof(float) + 1023) & ~1023u;
  float* buf = reinterpret_cast<float*>(smem + (ring - base)) + (size_t)warp * 4 * kTF;
  float* gx = static_cast<float*>(p.x);
  const long tiles = p.m;  // one system a tile
  const long first = (long)blockIdx.x * kWarps + warp;
  const long step = (long)gridDim.x * kWarps;
  if (lane == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncwarp();
  const auto issue = [&](long tile) {  // lane 0
    const int row = (int)(tile * (kTF / 32));
    mbar_arrive_expect_tx(bar, 4 * kTF * sizeof(float));
    tma_load_2d(buf + 0 * kTF, &ma, 0, row, bar);
    tma_load_2d(buf + 1 * kTF, &mb, 0, row, bar);
    tma_load_2d(buf + 2 * kTF, &mc, 0, row, bar);
    tma_load_2d(buf + 3 * kTF, &md, 0, row, bar);
  };
  if (lane == 0 && first < tiles) issue(first);
  int chunk[kR / 4];
#pragma unroll
  for (int q = 0; q < kR / 4; ++q) {
    const int c = lane * (kR / 4) + q, row = c >> 3;
    chunk[q] = row * 32 + (((c & 7) ^ (row & 7)) << 2);
  }
  int k = 0;
  for (long tile = first; tile < tiles; tile += step, ++k) {
    if (!mbar_wait(bar, k & 1, p.status)) break;
    float v[4][kR];
#pragma unroll
    for (int arr = 0; arr < 4; ++arr)
#pragma unroll
      for (int q = 0; q < kR / 4; ++q) {
        const float4 f = *reinterpret_cast<const float4*>(buf + arr * kTF + chunk[q]);
        v[arr][4 * q] = f.x; v[arr][4 * q + 1] = f.y; v[arr][4 * q + 2] = f.z; v[arr][4 * q + 3] = f.w;
      }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0 && tile + step < tiles) issue(tile + step);
    if (lane == 0) v[0][0] = 0.0f;          // a[0] is not part of the system
    if (lane == 31) v[2][kR - 1] = 0.0f;    // nor is c[n-1]
    // ---- CR level: odd rows 2j+1 against their even neighbours ----
    // (lane 31's last odd row has c = 0, so the shuffled-in neighbour, its
    // own first row, contributes nothing)
    const float ra = __shfl_down_sync(kFull, v[0][0], 1), rb = __shfl_down_sync(kFull, v[1][0], 1);
    const float rc = __shfl_down_sync(kFull, v[2][0], 1), rd = __shfl_down_sync(kFull, v[3][0], 1);
    NR2 P[kRR / 2];
#pragma unroll
    for (int j = 0; j < kRR; ++j) {
      const int q = 2 * j + 1;
      const float aR = q + 1 < kR ? v[0][q + 1] : ra, bR = q + 1 < kR ? v[1][q + 1] : rb;
      const float cR = q + 1 < kR ? v[2][q + 1] : rc, dR = q + 1 < kR ? v[3][q + 1] : rd;
      const float k1 = tdiv(v[0][q], v[1][q - 1]);
      const float k2 = tdiv(v[2][q], bR);
      const float an = -v[0][q - 1] * k1;
      const float bn = v[1][q] - v[2][q - 1] * k1 - aR * k2;
      const float cn = -cR * k2;
      const float dn = v[3][q] - v[3][q - 1] * k1 - dR * k2;
      const float ib = rcp_approx(bn);
      const NR r{an * ib, cn * ib, dn * ib};
      if (j & 1) {
        P[j / 2].a.y = r.a; P[j / 2].c.y = r.c; P[j / 2].d.y = r.d;
      } else {
        P[j / 2].a.x = r.a; P[j / 2].c.x = r.c; P[j / 2].d.x = r.d;
      }
    }
    // ---- PCR on the 512 intermediate rows (the two-phase kernel's n = 512 path) ----
    phase_a_pairs<kLPS, kRR>(P);
    transpose_word<kRR, kLPS>(sw, kRR * lane, lane, [&](int j) -> float2& { return P[j].a; });
    transpose_word<kRR, kLPS>(sw, kRR * lane, lane, [&](int j) -> float2& { return P[j].c; });
    transpose_word<kRR, kLPS>(sw, kRR * lane, lane, [&](int j) -> float2& { return P[j].d; });
    {
      NR w[kRR];
#pragma unroll
      for (int j = 0; j < kRR / 2; ++j) {
        w[2 * j] = row_x(P[j]);
        w[2 * j + 1] = row_y(P[j]);
      }
      phase_b_xor16<kRR>(w, lane);
      phase_b_step<1, kRR>(w);
#pragma unroll
      for (int j = 0; j < kRR / 2; ++j) P[j] = pair_of(w[2 * j], w[2 * j + 1]);
    }
    phase_b_pairs<2, kRR>(P);
    phase_b_pairs<4, kRR>(P);
    // ---- closing 2x2 systems (slots s, s + 8): x of intermediate row lane + 32 s ----
#pragma unroll
    for (int j = 0; j < kRR / 4; ++j) {
      const NR2& u = P[j];
      const NR2& l = P[j + kRR / 4];
      const float2 den = __ffma2_rn(neg2(u.c), l.a, make_float2(1.0f, 1.0f));
      const float2 num = __ffma2_rn(neg2(u.c), l.d, u.d);
      const float2 xu = __fmul2_rn(num, rcp_approx2(den));
      const float2 xl = __ffma2_rn(neg2(l.a), xu, l.d);
      sw[xr_index(lane + 32 * (2 * j))] = xu.x;
      sw[xr_index(lane + 32 * (2 * j + 1))] = xu.y;
      sw[xr_index(lane + 32 * (2 * j + kRR / 2))] = xl.x;
      sw[xr_index(lane + 32 * (2 * j + 1 + kRR / 2))] = xl.y;
    }
    __syncwarp();
    // ---- CR back substitution of the even rows; the lane's 32 unknowns out ----
    float xo[kR];
    float xprev = lane > 0 ? sw[xr_index(kRR * lane - 1)] : 0.0f;  // (row 0's a is zero)
#pragma unroll
    for (int j = 0; j < kRR; ++j) {
      const float xodd = sw[xr_index(kRR * lane + j)];
      const int q = 2 * j;
      xo[q] = (v[3][q] - v[0][q] * xprev - v[2][q] * xodd) * rcp_approx(v[1][q]);
      xo[q + 1] = xodd;
      xprev = xodd;
    }
    __syncwarp();  // the scratch is the next tile's transpose scratch
    if (tile < p.m) {
      float4* dst = reinterpret_cast<float4*>(gx + tile * kN + kR * lane);
#pragma unroll
      for (int q = 0; q < kR / 4; ++q) dst[q] = make_float4(xo[4 * q], xo[4 * q + 1], xo[4 * q + 2], xo[4 * q + 3]);
    }
  }
}

// One CR level of the lane's K unnormalised rows (local rows 0..K-1 of a
// contiguous block): the odd rows 2j+1 eliminate their even neighbours (the
// last one's right neighbour, row K of the block, is the next lane's row 0:
// one shuffle; lane 31's has c = 0 and contributes nothing).  The K/2 new
// rows land in (na, nb, nc, nd).
template <int K>
__device__ __forceinline__ void cr_level(const float (&a)[K], const float (&b)[K], const float (&c)[K],
                                         const float (&d)[K], float (&na)[K / 2], float (&nb)[K / 2],
                                         float (&nc)[K / 2], float (&nd)[K / 2]) {
  const float ra = __shfl_down_sync(kFull, a[0], 1), rb = __shfl_down_sync(kFull, b[0], 1);
  const float rc = __shfl_down_sync(kFull, c[0], 1), rd = __shfl_down_sync(kFull, d[0], 1);
#pragma unroll
  for (int j = 0; j < K / 2; ++j) {
    const int q = 2 * j + 1;
    const float aR = q + 1 < K ? a[q + 1] : ra, bR = q + 1 < K ? b[q + 1] : rb;
    const float cR = q + 1 < K ? c[q + 1] : rc, dR = q + 1 < K ? d[q + 1] : rd;
    const float k1 = tdiv(a[q], b[q - 1]);
    const float k2 = tdiv(c[q], bR);
    na[j] = -a[q - 1] * k1;
    nb[j] = b[q] - c[q - 1] * k1 - aR * k2;
    nc[j] = -cR * k2;
    nd[j] = d[q] - d[q - 1] * k1 - dR * k2;
  }
}

// The even rows of a CR level given x of the odd ones (xo[j] = x of row 2j+1
// of the lane's block): x[2j] = (d - a x[2j-1] - c x[2j+1]) / b, row -1 the
// previous lane's last odd row (zero for lane 0, whose first row has a = 0).
template <int K>
__device__ __forceinline__ void cr_back(const float (&a)[K], const float (&b)[K], const float (&c)[K],
                                        const float (&d)[K], const float (&xo)[K / 2], float (&x)[K], int lane) {
  float xprev = __shfl_up_sync(kFull, xo[K / 2 - 1], 1);
  if (lane == 0) xprev = 0.0f;
#pragma unroll
  for (int j = 0; j < K / 2; ++j) {
    x[2 * j] = (d[2 * j] - a[2 * j] * xprev - c[2 * j] * xo[j]) * rcp_approx(b[2 * j]);
    x[2 * j + 1] = xo[j];
    xprev = xo[j];
  }
}

constexpr int kS256 = 256 + 32;  // the 256-row PCR's scratch per word array (one pad word per 8 rows:
                                 // lane stride 9 words, conflict-free at every distance)
__device__ __forceinline__ int r256_index(int r) { return r + (r >> 3); }

// CR-PCR with the switch at n/4 for 1024 unknowns: two CR levels inside the
// lane (32 -> 16 -> 8 rows), PCR on the 256 rows left (distances 1, 2, 4
// inside the lane over shuffles, 8 .. 64 through the warp's scratch, the
// closing pairs (r, r + 128) over one xor-16 shuffle), the two back
// substitutions in the lane, 16-byte stores.
__global__ void __launch_bounds__(kWarps * 32, 3)
    crpcr256_kernel(HybridParams p, const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                    const __grid_constant__ CUtensorMap mc, const __grid_constant__ CUtensorMap md) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + warp;
  float* sw = reinterpret_cast<float*>(smem + 128) + (size_t)warp * 3 * kS256;
  const uint32_t base = smem_addr(smem);
  const uint32_t ring = (base + 128 + kWarps * 3 * kS256 * (uint32_t)sizeof(float) + 1023) & ~1023u;
  float* buf = reinterpret_cast<float*>(smem + (ring - base)) + (size_t)warp * 4 * kTF;
  float* gx = static_cast<float*>(p.x);
  const long tiles = p.m;
  const long first = (long)blockIdx.x * kWarps + warp;
  const long step = (long)gridDim.x * kWarps;
  if (lane == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncwarp();
  const auto issue = [&](long tile) {
    const int row = (int)(tile * (kTF / 32));
    mbar_arrive_expect_tx(bar, 4 * kTF * sizeof(float));
    tma_load_2d(buf + 0 * kTF, &ma, 0, row, bar);
    tma_load_2d(buf + 1 * kTF, &mb, 0, row, bar);
    tma_load_2d(buf + 2 * kTF, &mc, 0, row, bar);
    tma_load_2d(buf + 3 * kTF, &md, 0, row, bar);
  };
  if (lane == 0 && first < tiles) issue(first);
  int chunk[kR / 4];
#pragma unroll
  for (int q = 0; q < kR / 4; ++q) {
    const int c = lane * (kR / 4) + q, row = c >> 3;
    chunk[q] = row * 32 + (((c & 7) ^ (row & 7)) << 2);
  }
  float* sa = sw;
  float* sc = sw + kS256;
  float* sd = sw + 2 * kS256;
  int k = 0;
  for (long tile = first; tile < tiles; tile += step, ++k) {
    if (!mbar_wait(bar, k & 1, p.status)) break;
    float v[4][kR];
#pragma unroll
    for (int arr = 0; arr < 4; ++arr)
#pragma unroll
      for (int q = 0; q < kR / 4; ++q) {
        const float4 f = *reinterpret_cast<const float4*>(buf + arr * kTF + chunk[q]);
        v[arr][4 * q] = f.x; v[arr][4 * q + 1] = f.y; v[arr][4 * q + 2] = f.z; v[arr][4 * q + 3] = f.w;
      }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0 && tile + step < tiles) issue(tile + step);
    if (lane == 0) v[0][0] = 0.0f;
    if (lane == 31) v[2][kR - 1] = 0.0f;
    // ---- two CR levels inside the lane: 32 -> 16 -> 8 rows ----
    float a1[16], b1[16], c1[16], d1[16];
    cr_level<32>(v[0], v[1], v[2], v[3], a1, b1, c1, d1);
    float a2[8], b2[8], c2[8], d2[8];
    cr_level<16>(a1, b1, c1, d1, a2, b2, c2, d2);
    // ---- PCR on the 256 rows: lane t holds rows 8t .. 8t+7, normalised ----
    NR w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float ib = rcp_approx(b2[j]);
      w[j] = NR{a2[j] * ib, c2[j] * ib, d2[j] * ib};
    }
    phase_a_step<1, 32, 8>(w);
    phase_a_step<2, 32, 8>(w);
    phase_a_step<4, 32, 8>(w);
#pragma unroll
    for (int D = 8; D <= 64; D *= 2) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int r = 8 * lane + j;
        sa[r256_index(r)] = w[j].a;
        sc[r256_index(r)] = w[j].c;
        sd[r256_index(r)] = w[j].d;
      }
      __syncwarp();
      NR o[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int r = 8 * lane + j;
        // a neighbour beyond the system's ends: the row itself (its coupling there is exactly zero)
        const int il = r - D >= 0 ? r - D : r, ir = r + D < 256 ? r + D : r;
        const NR L{sa[r256_index(il)], sc[r256_index(il)], sd[r256_index(il)]};
        const NR Rr{sa[r256_index(ir)], sc[r256_index(ir)], sd[r256_index(ir)]};
        o[j] = step_both(w[j], L, Rr);
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 8; ++j) w[j] = o[j];
    }
    // ---- closing 2x2 systems (r, r + 128): lanes t and t ^ 16, same slot ----
    float x2[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const NR pr = shfl_xor_nr(w[j], 16);
      const NR& u = lane < 16 ? w[j] : pr;  // row r
      const NR& l = lane < 16 ? pr : w[j];  // row r + 128
      const float xu = (u.d - u.c * l.d) * rcp_approx(fmaf(-u.c, l.a, 1.0f));
      x2[j] = lane < 16 ? xu : fmaf(-l.a, xu, l.d);
    }
    // ---- CR back substitution: 8 -> 16 -> 32 rows ----
    float x1[16], x[kR];
    cr_back<16>(a1, b1, c1, d1, x2, x1, lane);
    cr_back<32>(v[0], v[1], v[2], v[3], x1, x, lane);
    if (tile < p.m) {
      float4* dst = reinterpret_cast<float4*>(gx + tile * kN + kR * lane);
#pragma unroll
      for (int q = 0; q < kR / 4; ++q) dst[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
    }
  }
}

}  // namespace

// True when a register kernel takes this FP32 call: crpcr with rest = n/2
// or n/4 at n = 1024, 16-byte aligned a..d and x, the batch within the tensor
// maps' 32-bit row count.
bool crpcr1024_applies(const void* a, const void* b, const void* c, const void* d, const void* x, int n, long m,
                       int stride) {
  return n == kN && (stride == 2 || stride == 4) && aligned16(a) && aligned16(b) && aligned16(c) && aligned16(d) &&
         aligned16(x) && m * n / 32 < (1L << 31) && tunable(TRIDI_TUNE_PCR_KERNEL) != 2 && !g_host_mapped_io;
}

tridi_status crpcr1024_solve(const float* a, const float* b, const float* c, const float* d, float* x, int m,
                             int stride, cudaStream_t stream) {
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  HybridParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = kN; p.m = m; p.stride = stride;
  p.status = dev->status;
  const uint64_t rows = (uint64_t)m * kN / 32;
  CUtensorMap tma, tmb, tmc, tmd;
  if (!make_tensor_map_2d(&tma, a, 32, rows, 128, 32, kR, true) ||
      !make_tensor_map_2d(&tmb, b, 32, rows, 128, 32, kR, true) ||
      !make_tensor_map_2d(&tmc, c, 32, rows, 128, 32, kR, true) ||
      !make_tensor_map_2d(&tmd, d, 32, rows, 128, 32, kR, true))
    return cuda_status(cudaErrorInvalidValue);
  const auto kern = stride == 2 ? crpcr512_kernel : crpcr256_kernel;
  const size_t smem = stride == 2 ? kSmem : kSmem256;
  if (smem > (size_t)dev->max_smem_optin) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
  if (e != cudaSuccess) return cuda_status(e);
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev->sm_count;
  if (grid * kWarps > m) grid = (m + kWarps - 1) / kWarps;
  kern<<<(unsigned)grid, kWarps * 32, smem, stream>>>(p, tma, tmb, tmc, tmd);
  return cuda_status(cudaGetLastError());
}

}  // namespace tridi

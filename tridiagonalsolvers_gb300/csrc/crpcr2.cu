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

}  // namespace

// True when the register kernel takes this FP32 call: crpcr with rest = n/2
// at n = 1024, 16-byte aligned a..d and x, the batch within the tensor maps'
// 32-bit row count.
bool crpcr512_applies(const void* a, const void* b, const void* c, const void* d, const void* x, int n, long m,
                      int stride) {
  return n == kN && stride == 2 && aligned16(a) && aligned16(b) && aligned16(c) && aligned16(d) && aligned16(x) &&
         m * n / 32 < (1L << 31) && tunable(TRIDI_TUNE_PCR_KERNEL) != 2 && !g_host_mapped_io;
}

tridi_status crpcr512_solve(const float* a, const float* b, const float* c, const float* d, float* x, int m,
                            cudaStream_t stream) {
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  HybridParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = kN; p.m = m; p.stride = 2;
  p.status = dev->status;
  const uint64_t rows = (uint64_t)m * kN / 32;
  CUtensorMap tma, tmb, tmc, tmd;
  if (!make_tensor_map_2d(&tma, a, 32, rows, 128, 32, kR, true) ||
      !make_tensor_map_2d(&tmb, b, 32, rows, 128, 32, kR, true) ||
      !make_tensor_map_2d(&tmc, c, 32, rows, 128, 32, kR, true) ||
      !make_tensor_map_2d(&tmd, d, 32, rows, 128, 32, kR, true))
    return cuda_status(cudaErrorInvalidValue);
  if (kSmem > (size_t)dev->max_smem_optin) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  cudaError_t e = cudaFuncSetAttribute(crpcr512_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (e != cudaSuccess) return cuda_status(e);
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, crpcr512_kernel, kWarps * 32, kSmem);
  if (e != cudaSuccess) return cuda_status(e);
  if (per_sm < 1) per_sm = 1;
  long grid = (long)per_sm * dev->sm_count;
  if (grid * kWarps > m) grid = (m + kWarps - 1) / kWarps;
  crpcr512_kernel<<<(unsigned)grid, kWarps * 32, kSmem, stream>>>(p, tma, tmb, tmc, tmd);
  return cuda_status(cudaGetLastError());
}

}  // namespace tridi

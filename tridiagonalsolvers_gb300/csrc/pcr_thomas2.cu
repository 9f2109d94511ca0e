// PCR-then-Thomas ("pcrGauss", pcrGauss_kernel.cu:1-126, pcrGauss_app.cu:164)
// for FP32 systems of 64..1024 unknowns (power of two) in registers, on the
// two-phase layout of pcr_twophase.cuh.
//
// log2(G) PCR steps (distances 1, 2, ..., G/2) leave G independent chains of
// stride G (rows c, c + G, c + 2G, ...); each chain is then solved by Thomas.
// The PCR steps are those of the two-phase kernel: distances up to R/2 on the
// lane's R contiguous rows (phase A), then, after the transpose that gives
// lane t the rows t + LPS*s, the larger distances on the slot index (phase
// B).  In that layout chain c lies entirely in lane c mod LPS (for G a
// multiple of LPS): lane t holds the G/LPS chains t + LPS*s0, s0 < G/LPS, in
// slots s0, s0 + G/LPS, s0 + 2G/LPS, ...  So the Thomas sweeps run in the
// lane's registers, two chains per paired FP32 instruction where a lane holds
// more than one, and x leaves from them as the two-phase kernel's does.
//
// G is the caller's split g where g >= LPS.  A smaller g would leave chains
// spread over several lanes; there G = LPS: the extra PCR steps keep the
// solution exact (after any number of PCR steps the chains solve the same
// system), and only the rounding differs from a split into g chains.  (The
// reference's own tables often take fewer steps than log2(g), and its result
// is then an approximation: pcrGauss_app.cu:12-96.)
#include "hybrid.cuh"
#include "pcr_twophase.cuh"
#include "runtime.h"

namespace tridi {

namespace {

using namespace pcr2;

// Thomas on the lane's chains: KG chains of R / KG rows, chain s0 in slots
// s0 + KG * k (normalised rows: a x_prev + x + c x_next = d).  dst: the
// lane's first unknown; slot s is unknown LPS * s.
template <int R, int KG, int LPS>
__device__ __forceinline__ void thomas_pairs(NR2 (&P)[R / 2], float* dst, bool store) {
  constexpr int KP = KG / 2;  // chain pairs (slots 2 j', 2 j' + 1 of pair j')
  constexpr int L = R / KG;   // rows per chain
#pragma unroll
  for (int jp = 0; jp < KP; ++jp) {
    float2 cp = P[jp].c, dp = P[jp].d;
#pragma unroll
    for (int k = 1; k < L; ++k) {
      NR2& r = P[jp + KP * k];
      const float2 na = neg2(r.a);
      const float2 inv = rcp_approx2(__ffma2_rn(na, cp, make_float2(1.0f, 1.0f)));
      cp = __fmul2_rn(r.c, inv);
      dp = __fmul2_rn(__ffma2_rn(na, dp, r.d), inv);
      r.c = cp;
      r.d = dp;
    }
    float2 x = dp;
#pragma unroll
    for (int k = L - 1; k >= 0; --k) {
      const int j = jp + KP * k;
      if (k < L - 1) x = __ffma2_rn(neg2(P[j].c), x, P[j].d);
      if (store) {
        dst[LPS * (2 * j)] = x.x;
        dst[LPS * (2 * j + 1)] = x.y;
      }
    }
  }
}

// One chain a lane (G = LPS): slots 0 .. R-1 in order.
template <int R, int LPS>
__device__ __forceinline__ void thomas_single(NR (&w)[R], float* dst, bool store) {
  float cp = w[0].c, dp = w[0].d;
#pragma unroll
  for (int s = 1; s < R; ++s) {
    const float inv = rcp_approx(fmaf(-w[s].a, cp, 1.0f));
    cp = w[s].c * inv;
    dp = fmaf(-w[s].a, dp, w[s].d) * inv;
    w[s].c = cp;
    w[s].d = dp;
  }
  float x = dp;
  if (store) dst[LPS * (R - 1)] = x;
#pragma unroll
  for (int s = R - 2; s >= 0; --s) {
    x = fmaf(-w[s].c, x, w[s].d);
    if (store) dst[LPS * s] = x;
  }
}

// One launch: every warp streams its own tiles of 32/LPS systems (the tile
// pipeline of pcr_twophase_kernel).
template <int N, int G>
__global__ void __launch_bounds__(Pcr2Shape<N>::WARPS * 32, 3)
    pcr_thomas2_kernel(HybridParams p, const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                       const __grid_constant__ CUtensorMap mc, const __grid_constant__ CUtensorMap md) {
  using S = Pcr2Shape<N>;
  constexpr int R = S::R, LPS = S::LPS, SPW = S::SPW, TF = S::TF;
  constexpr int BUF = 4 * TF;
  constexpr int SYS_STRIDE = S::SYS_STRIDE;
  constexpr int KG = G / LPS;  // chains a lane
  static_assert(N >= 64 && N <= 1024 && SPW * N == TF, "pcr_thomas2: 64 <= n <= 1024");
  static_assert(G >= LPS && G % LPS == 0 && G <= N / 4 && (KG == 1 || KG % 2 == 0), "pcr_thomas2: split");
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + warp;
  float* scratch = reinterpret_cast<float*>(smem + 128) + (size_t)warp * S::SCRATCH;
  const uint32_t base = smem_addr(smem);
  const uint32_t ring = (base + 128 + S::WARPS * S::SCRATCH * (uint32_t)sizeof(float) + 1023) & ~1023u;
  float* buf = reinterpret_cast<float*>(smem + (ring - base)) + (size_t)warp * BUF;
  float* gx = static_cast<float*>(p.x);
  const long tiles = ((long)p.m + SPW - 1) / SPW;
  const long first = (long)blockIdx.x * (blockDim.x >> 5) + warp;
  const long step = (long)gridDim.x * (blockDim.x >> 5);
  if (lane == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncwarp();
  const auto issue = [&](long tile) {  // lane 0; the last tile's box reads zeros beyond the batch
    const int row = (int)(tile * (TF / 32));
    mbar_arrive_expect_tx(bar, 4 * TF * sizeof(float));
    tma_load_2d(buf + 0 * TF, &ma, 0, row, bar);
    tma_load_2d(buf + 1 * TF, &mb, 0, row, bar);
    tma_load_2d(buf + 2 * TF, &mc, 0, row, bar);
    tma_load_2d(buf + 3 * TF, &md, 0, row, bar);
  };
  if (lane == 0 && first < tiles) issue(first);
  const int g = lane / LPS, t = lane % LPS;
  int chunk[R / 4];
#pragma unroll
  for (int q = 0; q < R / 4; ++q) {
    const int c = lane * (R / 4) + q, row = c >> 3;
    chunk[q] = row * 32 + (((c & 7) ^ (row & 7)) << 2);
  }
  int k = 0;
  for (long tile = first; tile < tiles; tile += step, ++k) {
    if (!mbar_wait(bar, k & 1, p.status)) break;
    float v[4][R];
#pragma unroll
    for (int arr = 0; arr < 4; ++arr)
#pragma unroll
      for (int q = 0; q < R / 4; ++q) {
        const float4 f = *reinterpret_cast<const float4*>(buf + arr * TF + chunk[q]);
        v[arr][4 * q] = f.x; v[arr][4 * q + 1] = f.y; v[arr][4 * q + 2] = f.z; v[arr][4 * q + 3] = f.w;
      }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0 && tile + step < tiles) issue(tile + step);
    if (t == 0) v[0][0] = 0.0f;            // a[0] is not part of the system
    if (t == LPS - 1) v[2][R - 1] = 0.0f;  // nor is c[n-1]
    float* sw = scratch + g * SYS_STRIDE;
    const int rb = t * R;
    const long sys = tile * SPW + g;
    float* dst = gx + sys * N + t;
    const bool store = sys < p.m;
    NR2 P[R / 2];
#pragma unroll
    for (int j = 0; j < R / 2; ++j) {
      const float2 ib = rcp_approx2(make_float2(v[1][2 * j], v[1][2 * j + 1]));
      P[j] = NR2{__fmul2_rn(make_float2(v[0][2 * j], v[0][2 * j + 1]), ib),
                 __fmul2_rn(make_float2(v[2][2 * j], v[2][2 * j + 1]), ib),
                 __fmul2_rn(make_float2(v[3][2 * j], v[3][2 * j + 1]), ib)};
    }
    // ---- phase A: distances 1 .. min(G, R) / 2 ----
    phase_a_step1_pairs<LPS, R>(P);
    if constexpr (2 <= G / 2) phase_a_step_pairs<1, LPS, R>(P);
    if constexpr (4 <= G / 2) phase_a_step_pairs<2, LPS, R>(P);
    if constexpr (8 <= G / 2 && 8 <= R / 2) phase_a_step_pairs<4, LPS, R>(P);
    if constexpr (16 <= G / 2 && 16 <= R / 2) phase_a_step_pairs<8, LPS, R>(P);
    // ---- transpose: lane t of system g takes rows t + LPS * s ----
    transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].a; });
    transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].c; });
    transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].d; });
    // ---- phase B: distances R .. G/2 ----
    if constexpr (N == 512) {  // distance 16 (= R) is the lane exchange c ^ 16; G >= LPS = 32
      NR w[R];
#pragma unroll
      for (int j = 0; j < R / 2; ++j) {
        w[2 * j] = row_x(P[j]);
        w[2 * j + 1] = row_y(P[j]);
      }
      phase_b_xor16<R>(w, lane);
      if constexpr (G >= 64) phase_b_step<1, R>(w);
#pragma unroll
      for (int j = 0; j < R / 2; ++j) P[j] = pair_of(w[2 * j], w[2 * j + 1]);
      if constexpr (G >= 128) phase_b_pairs<2, R>(P);
    } else {
      if constexpr (R <= G / 2) phase_b_pairs<R / LPS, R>(P);
      if constexpr (2 * R <= G / 2) phase_b_pairs<2 * R / LPS, R>(P);
      if constexpr (4 * R <= G / 2) phase_b_pairs<4 * R / LPS, R>(P);
    }
    // ---- Thomas on the lane's chains ----
    if constexpr (KG == 1) {
      NR w[R];
#pragma unroll
      for (int j = 0; j < R / 2; ++j) {
        w[2 * j] = row_x(P[j]);
        w[2 * j + 1] = row_y(P[j]);
      }
      thomas_single<R, LPS>(w, dst, store);
    } else {
      thomas_pairs<R, KG, LPS>(P, dst, store);
    }
  }
}

template <int N, int G>
cudaError_t launch_pcr_thomas2(const HybridParams& p, const DeviceInfo& dev, cudaStream_t stream) {
  using S = Pcr2Shape<N>;
  auto kern = pcr_thomas2_kernel<N, G>;
  constexpr int kThreads = S::WARPS * 32;
  const uint64_t rows = (uint64_t)p.m * N / 32;
  CUtensorMap ma, mb, mc, md;
  if (!make_tensor_map_2d(&ma, static_cast<const float*>(p.a), 32, rows, 128, 32, S::R, true) ||
      !make_tensor_map_2d(&mb, static_cast<const float*>(p.b), 32, rows, 128, 32, S::R, true) ||
      !make_tensor_map_2d(&mc, static_cast<const float*>(p.c), 32, rows, 128, 32, S::R, true) ||
      !make_tensor_map_2d(&md, static_cast<const float*>(p.d), 32, rows, 128, 32, S::R, true))
    return cudaErrorInvalidValue;
  if (S::SMEM > (size_t)dev.max_smem_optin) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, S::SMEM);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const long tiles = ((long)p.m + S::SPW - 1) / S::SPW;
  long grid = (long)per_sm * dev.sm_count;
  if (grid * S::WARPS > tiles) grid = (tiles + S::WARPS - 1) / S::WARPS;
  kern<<<(unsigned)grid, kThreads, S::SMEM, stream>>>(p, ma, mb, mc, md);
  return cudaGetLastError();
}

// G from the caller's g (raised to LPS), for n and G with an instantiated kernel.
template <int N>
cudaError_t launch_for_n(const HybridParams& p, int g, const DeviceInfo& dev, cudaStream_t stream) {
  constexpr int LPS = Pcr2Shape<N>::LPS;
  const int G = g < LPS ? LPS : g;
  switch (G / LPS) {
    case 1: return launch_pcr_thomas2<N, LPS>(p, dev, stream);
    case 2: if constexpr (2 * LPS <= N / 4) return launch_pcr_thomas2<N, 2 * LPS>(p, dev, stream); break;
    case 4: if constexpr (4 * LPS <= N / 4) return launch_pcr_thomas2<N, 4 * LPS>(p, dev, stream); break;
    case 8: if constexpr (8 * LPS <= N / 4) return launch_pcr_thomas2<N, 8 * LPS>(p, dev, stream); break;
    default: break;
  }
  return cudaErrorInvalidValue;
}

}  // namespace

// True when the register kernel takes this FP32 call: n a power of two in
// 64 .. 1024, g < n/2 (g >= n/2 is the full PCR kernel's), 16-byte aligned
// contiguous arrays, the batch within the tensor maps' 32-bit row count.
bool pcr_thomas2_applies(const void* a, const void* b, const void* c, const void* d, int n, long m, int g) {
  return (n == 64 || n == 128 || n == 256 || n == 512 || n == 1024) && g >= 1 && g < n / 2 && aligned16(a) &&
         aligned16(b) && aligned16(c) && aligned16(d) && m * n / 32 < (1L << 31) &&
         tunable(TRIDI_TUNE_PCR_KERNEL) != 2 && !g_host_mapped_io;
}

tridi_status pcr_thomas2_solve(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                               int m, int g, cudaStream_t stream) {
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  HybridParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.stride = 1;
  p.status = dev->status;
  cudaError_t e = cudaErrorInvalidValue;
  switch (n) {
    case 64: e = launch_for_n<64>(p, g, *dev, stream); break;
    case 128: e = launch_for_n<128>(p, g, *dev, stream); break;
    case 256: e = launch_for_n<256>(p, g, *dev, stream); break;
    case 512: e = launch_for_n<512>(p, g, *dev, stream); break;
    case 1024: e = launch_for_n<1024>(p, g, *dev, stream); break;
    default: break;
  }
  return cuda_status(e);
}

}  // namespace tridi

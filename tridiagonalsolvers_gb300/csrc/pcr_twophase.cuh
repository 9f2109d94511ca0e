// Parallel cyclic reduction for FP32 systems of 64..1024 unknowns in two
// register phases around one transpose (replaces the device work of pcr(),
// pcr_app.cu:5 / pcrKernel, pcr_kernel.cu:1-77, at these sizes).
//
// The algorithm is the reference's: log2(n/2) PCR steps with distances
// 1, 2, ..., n/4, each eliminating every row's couplings against its
// neighbours at that distance, then n/2 independent 2x2 systems (i, i+n/2).
// Rows are kept normalised (divided by their diagonal, b = 1): each step
// forms me - a*L - c*R from the normalised neighbours L, R and normalises the
// result with one reciprocal, so three words per row move between lanes and
// each row costs one reciprocal per step.
//
// Mapping (R rows a lane: 16 up to n = 512, 32 at n = 1024; n = R * LPS,
// LPS lanes per system, 32 / LPS systems per warp):
//   phase A  lane p holds rows R p .. R p + R-1.  Steps of distance 1 .. R/2
//            run inside the lane; a row whose neighbour lies in the next or
//            previous lane gets it over one shuffle (3 words).
//   transpose  the normalised rows go through the warp's staging buffer
//            (16-byte stores, XOR-swizzled so that neither the stores nor the
//            4-byte loads of the other side conflict on banks), and lane c
//            takes rows c + LPS*s, s = 0 .. R-1.
//   phase B  distances R .. n/4 move only the slot index s and stay inside
//            the lane (n = 512: distance 16 is a lane exchange with lane
//            c ^ 16); neighbours beyond the system's ends have coupling
//            exactly zero and are skipped at compile time.  The closing 2x2
//            systems pair slots s and s + R/2 of the same lane.
// x is written straight from phase B: for a fixed s the LPS lanes of a system
// store LPS consecutive unknowns.
// The steps whose neighbours are whole row pairs (rows 2j, 2j+1) -- all but
// distance 1 and slot distance 1 -- run two rows per paired FP32 instruction
// (FFMA2 / FMUL2, sm_100+).
// Input rows arrive through one staging buffer per warp: a tile (32/LPS
// systems, 32 R consecutive values of each array) is one R x 128-byte box of
// each array's tensor map, copied by cp.async.bulk.tensor with the 128-byte
// swizzle, so the 16-byte loads of a lane's 4 R bytes are conflict-free with
// no register shuffling (16-byte chunk c of box row r is stored at chunk
// c ^ (r mod 8)).  As soon as a tile is in registers the warp issues the
// next one into the same buffer: its load has the whole solve of this tile
// to land, and one buffer per warp (plus a transpose scratch of one word
// array) lets more warps share an SM.
#pragma once
#include "tridi_device.cuh"

namespace tridi {

namespace pcr2 {

// One normalised row: a x[i-dl] + x[i] + c x[i+dl] = d.
struct NR {
  float a, c, d;
};

__device__ __forceinline__ float2 rcp_approx2(float2 v) { return make_float2(rcp_approx(v.x), rcp_approx(v.y)); }

// me - me.a * L - me.c * R, normalised.
__device__ __forceinline__ NR step_both(const NR& me, const NR& L, const NR& R) {
  const float b = fmaf(-me.c, R.a, fmaf(-me.a, L.c, 1.0f));
  const float d = fmaf(-me.c, R.d, fmaf(-me.a, L.d, me.d));
  const float ib = rcp_approx(b);
  return {(-me.a * L.a) * ib, (-me.c * R.c) * ib, d * ib};
}
// The left neighbour lies beyond the system's first row: its coupling me.a is
// exactly zero.
__device__ __forceinline__ NR step_right(const NR& me, const NR& R) {
  const float b = fmaf(-me.c, R.a, 1.0f);
  const float d = fmaf(-me.c, R.d, me.d);
  const float ib = rcp_approx(b);
  return {0.0f, (-me.c * R.c) * ib, d * ib};
}
// The right neighbour lies beyond the system's last row.
__device__ __forceinline__ NR step_left(const NR& me, const NR& L) {
  const float b = fmaf(-me.a, L.c, 1.0f);
  const float d = fmaf(-me.a, L.d, me.d);
  const float ib = rcp_approx(b);
  return {(-me.a * L.a) * ib, 0.0f, d * ib};
}

// Two rows at once (components x, y).
struct NR2 {
  float2 a, c, d;
};
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ NR2 step_both2(const NR2& me, const NR2& L, const NR2& R) {
  const float2 na = neg2(me.a), nc = neg2(me.c);
  const float2 b = __ffma2_rn(nc, R.a, __ffma2_rn(na, L.c, make_float2(1.0f, 1.0f)));
  const float2 d = __ffma2_rn(nc, R.d, __ffma2_rn(na, L.d, me.d));
  const float2 ib = rcp_approx2(b);
  return {__fmul2_rn(__fmul2_rn(na, L.a), ib), __fmul2_rn(__fmul2_rn(nc, R.c), ib), __fmul2_rn(d, ib)};
}
__device__ __forceinline__ NR2 step_right2(const NR2& me, const NR2& R) {
  const float2 nc = neg2(me.c);
  const float2 b = __ffma2_rn(nc, R.a, make_float2(1.0f, 1.0f));
  const float2 d = __ffma2_rn(nc, R.d, me.d);
  const float2 ib = rcp_approx2(b);
  return {make_float2(0.0f, 0.0f), __fmul2_rn(__fmul2_rn(nc, R.c), ib), __fmul2_rn(d, ib)};
}
__device__ __forceinline__ NR2 step_left2(const NR2& me, const NR2& L) {
  const float2 na = neg2(me.a);
  const float2 b = __ffma2_rn(na, L.c, make_float2(1.0f, 1.0f));
  const float2 d = __ffma2_rn(na, L.d, me.d);
  const float2 ib = rcp_approx2(b);
  return {__fmul2_rn(__fmul2_rn(na, L.a), ib), make_float2(0.0f, 0.0f), __fmul2_rn(d, ib)};
}
__device__ __forceinline__ NR row_x(const NR2& v) { return {v.a.x, v.c.x, v.d.x}; }
__device__ __forceinline__ NR row_y(const NR2& v) { return {v.a.y, v.c.y, v.d.y}; }
__device__ __forceinline__ NR2 pair_of(const NR& x, const NR& y) {
  return {make_float2(x.a, y.a), make_float2(x.c, y.c), make_float2(x.d, y.d)};
}

__device__ __forceinline__ NR shfl_up_nr(const NR& v, int width) {
  return {__shfl_up_sync(kFull, v.a, 1, width), __shfl_up_sync(kFull, v.c, 1, width),
          __shfl_up_sync(kFull, v.d, 1, width)};
}
__device__ __forceinline__ NR shfl_down_nr(const NR& v, int width) {
  return {__shfl_down_sync(kFull, v.a, 1, width), __shfl_down_sync(kFull, v.c, 1, width),
          __shfl_down_sync(kFull, v.d, 1, width)};
}
__device__ __forceinline__ NR shfl_xor_nr(const NR& v, int mask) {
  return {__shfl_xor_sync(kFull, v.a, mask), __shfl_xor_sync(kFull, v.c, mask), __shfl_xor_sync(kFull, v.d, mask)};
}
__device__ __forceinline__ NR2 shfl_up_nr2(const NR2& v, int width) {
  return pair_of(shfl_up_nr(row_x(v), width), shfl_up_nr(row_y(v), width));
}
__device__ __forceinline__ NR2 shfl_down_nr2(const NR2& v, int width) {
  return pair_of(shfl_down_nr(row_x(v), width), shfl_down_nr(row_y(v), width));
}

// ---- single rows ------------------------------------------------------------
// Phase A step of distance DL (1 .. R/2) on the lane's contiguous rows.  Rows
// are visited by residue j mod DL, so each old row dies right after its last
// use.  Lanes at the system's ends receive their own row from the shuffle:
// its coupling there is exactly zero (a[0] = c[n-1] = 0 and, by induction
// over the steps, every row closer to an end than the step distance).
template <int DL, int LPS, int R>
__device__ __forceinline__ void phase_a_step(NR (&w)[R]) {
  NR o[R];
#pragma unroll
  for (int j = 0; j < DL; ++j) {
    const NR fromL = shfl_up_nr(w[R - DL + j], LPS);  // previous lane's row R-DL+j
    const NR fromR = shfl_down_nr(w[j], LPS);         // next lane's row j
#pragma unroll
    for (int q = j; q < R; q += DL) {
      const NR& L = q >= DL ? w[q - DL] : fromL;
      const NR& Rr = q + DL < R ? w[q + DL] : fromR;
      o[q] = step_both(w[q], L, Rr);
    }
  }
#pragma unroll
  for (int q = 0; q < R; ++q) w[q] = o[q];
}

// Phase B step moving the slot index by K (rows c + LPS*s: distance K*LPS).
template <int K, int R>
__device__ __forceinline__ void phase_b_step(NR (&w)[R]) {
  NR o[R];
#pragma unroll
  for (int s = 0; s < R; ++s) {
    if (s >= K && s + K < R) o[s] = step_both(w[s], w[s - K], w[s + K]);
    else if (s + K < R) o[s] = step_right(w[s], w[s + K]);
    else o[s] = step_left(w[s], w[s - K]);
  }
#pragma unroll
  for (int s = 0; s < R; ++s) w[s] = o[s];
}

// n = 512 only: distance 16 after the transpose (lane c holds rows c + 32 s):
// the neighbours at +-16 are lane c ^ 16, in slot s (the nearer side) or
// s -/+ 1 (the farther side).
template <int R>
__device__ __forceinline__ void phase_b_xor16(NR (&w)[R], int lane) {
  NR px[R];
#pragma unroll
  for (int s = 0; s < R; ++s) px[s] = shfl_xor_nr(w[s], 16);
  const bool lower = lane < 16;  // row c + 32 s, c < 16: R = partner slot s, L = partner slot s-1
  NR o[R];
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const NR Lf = s > 0 ? px[s - 1] : w[s];      // (beyond the first row when s = 0: coupling zero)
    const NR Rf = s + 1 < R ? px[s + 1] : w[s];  // (beyond the last row)
    const NR L = lower ? Lf : px[s];
    const NR Rr = lower ? px[s] : Rf;
    o[s] = step_both(w[s], L, Rr);
  }
#pragma unroll
  for (int s = 0; s < R; ++s) w[s] = o[s];
}

// ---- row pairs P[j] = rows (2j, 2j+1) -------------------------------------
// Distance 1 (phase A) and slot distance 1 (phase B) pair a row with halves
// of two different pairs; those steps run on single rows.
template <int LPS, int R>
__device__ __forceinline__ void phase_a_step1_pairs(NR2 (&P)[R / 2]) {
  constexpr int NP = R / 2;
  const NR fromL = shfl_up_nr(row_y(P[NP - 1]), LPS);  // previous lane's last row
  const NR fromR = shfl_down_nr(row_x(P[0]), LPS);     // next lane's first row
  NR2 o[NP];
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    const NR lo = step_both(row_x(P[j]), j > 0 ? row_y(P[j - 1]) : fromL, row_y(P[j]));
    const NR hi = step_both(row_y(P[j]), row_x(P[j]), j + 1 < NP ? row_x(P[j + 1]) : fromR);
    o[j] = pair_of(lo, hi);
  }
#pragma unroll
  for (int j = 0; j < NP; ++j) P[j] = o[j];
}
// Distance 2*DP rows (DP whole pairs) on contiguous rows.
template <int DP, int LPS, int R>
__device__ __forceinline__ void phase_a_step_pairs(NR2 (&P)[R / 2]) {
  constexpr int NP = R / 2;
  NR2 o[NP];
#pragma unroll
  for (int j = 0; j < DP; ++j) {
    const NR2 fromL = shfl_up_nr2(P[NP - DP + j], LPS);  // previous lane's pair NP-DP+j
    const NR2 fromR = shfl_down_nr2(P[j], LPS);          // next lane's pair j
#pragma unroll
    for (int q = j; q < NP; q += DP) {
      const NR2& L = q >= DP ? P[q - DP] : fromL;
      const NR2& Rr = q + DP < NP ? P[q + DP] : fromR;
      o[q] = step_both2(P[q], L, Rr);
    }
  }
#pragma unroll
  for (int q = 0; q < NP; ++q) P[q] = o[q];
}
template <int R>
__device__ __forceinline__ void phase_b_step1_pairs(NR2 (&P)[R / 2]) {
  constexpr int NP = R / 2;
  NR2 o[NP];
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    const NR lo = j > 0 ? step_both(row_x(P[j]), row_y(P[j - 1]), row_y(P[j])) : step_right(row_x(P[j]), row_y(P[j]));
    const NR hi = j + 1 < NP ? step_both(row_y(P[j]), row_x(P[j]), row_x(P[j + 1]))
                             : step_left(row_y(P[j]), row_x(P[j]));
    o[j] = pair_of(lo, hi);
  }
#pragma unroll
  for (int j = 0; j < NP; ++j) P[j] = o[j];
}
// Slot distance 2*DP (DP whole pairs).
template <int DP, int R>
__device__ __forceinline__ void phase_b_step_pairs(NR2 (&P)[R / 2]) {
  constexpr int NP = R / 2;
  NR2 o[NP];
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    if (j >= DP && j + DP < NP) o[j] = step_both2(P[j], P[j - DP], P[j + DP]);
    else if (j + DP < NP) o[j] = step_right2(P[j], P[j + DP]);
    else o[j] = step_left2(P[j], P[j - DP]);
  }
#pragma unroll
  for (int j = 0; j < NP; ++j) P[j] = o[j];
}

// Phase A on row pairs: distance 1, then 2 .. R/2 (whole pairs).
template <int LPS, int R>
__device__ __forceinline__ void phase_a_pairs(NR2 (&P)[R / 2]) {
  phase_a_step1_pairs<LPS, R>(P);
  phase_a_step_pairs<1, LPS, R>(P);
  phase_a_step_pairs<2, LPS, R>(P);
  phase_a_step_pairs<4, LPS, R>(P);
  if constexpr (R >= 32) phase_a_step_pairs<8, LPS, R>(P);
}
// Phase B on row pairs, slot distance K.
template <int K, int R>
__device__ __forceinline__ void phase_b_pairs(NR2 (&P)[R / 2]) {
  if constexpr (K == 1) phase_b_step1_pairs<R>(P);
  else phase_b_step_pairs<K / 2, R>(P);
}

// Scratch index of row r of one system's word array.  The R rows of phase-A
// lane p = r / R form a block of R/4 16-byte chunks, XOR-swizzled so that the
// 16-byte stores of 8 consecutive lanes and the 4-byte loads of rows
// c + LPS s (fixed s, consecutive c) each fall on distinct banks.
template <int R>
__device__ __forceinline__ int swz(int r) {
  const int p = r / R, j = r % R;
  if constexpr (R == 16) return (p << 4) + ((((j >> 2) ^ (p >> 1)) & 3) << 2) + (j & 3);
  else return (p << 5) + ((((j >> 2) ^ p) & 7) << 2) + (j & 3);
}

// One word array of the transpose through the warp's scratch: the lane's
// phase-A rows rb .. rb+R-1 go out as 16-byte stores, rows t + LPS*s come
// back (word(j) is the pair of rows 2j, 2j+1 before and slots 2j, 2j+1
// after).  The warp synchronises before the loads and after them (the next
// word array reuses the scratch).
template <int R, int LPS, class Word>
__device__ __forceinline__ void transpose_word(float* sw, int rb, int t, Word word) {
#pragma unroll
  for (int q4 = 0; q4 < R / 4; ++q4) {
    const float2 u = word(2 * q4), h = word(2 * q4 + 1);
    *reinterpret_cast<float4*>(sw + swz<R>(rb + 4 * q4)) = make_float4(u.x, u.y, h.x, h.y);
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < R / 2; ++j) word(j) = make_float2(sw[swz<R>(t + LPS * (2 * j))], sw[swz<R>(t + LPS * (2 * j + 1))]);
  __syncwarp();
}

}  // namespace pcr2

// Shared memory of one CTA: barriers, the transpose scratch of every warp
// (one word array of its tile, padded per system), then (1024-byte aligned,
// as the 128-byte swizzle requires) one staging buffer per warp of 4 arrays
// x 32 R values.
template <int N>
struct Pcr2Shape {
  static constexpr int R = N >= 1024 ? 32 : 16;  // rows a lane holds
  static constexpr int LPS = N / R;              // lanes per system
  static constexpr int SPW = 32 / LPS;           // systems per warp tile
  static constexpr int TF = 32 * R;              // values of one array in a warp tile (= SPW * N)
  static constexpr int WARPS = R == 32 ? 2 : 4;  // warps per CTA
  static constexpr int SYS_STRIDE = N + LPS;     // transpose scratch per system (padded: no bank conflicts)
  static constexpr int SCRATCH = SPW * SYS_STRIDE;  // floats per warp
  static constexpr size_t SMEM = 128 + (size_t)WARPS * SCRATCH * sizeof(float) + 1024 +
                                 (size_t)WARPS * 4 * TF * sizeof(float);
};

// One launch: every warp streams its own tiles of 32/LPS systems.  PAIRED:
// the steps whose neighbours are whole row pairs run two rows per
// instruction; otherwise every step runs on single rows.
template <int N, bool PAIRED>
__global__ void __launch_bounds__(Pcr2Shape<N>::WARPS * 32, 3)
    pcr_twophase_kernel(HybridParams p, const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                        const __grid_constant__ CUtensorMap mc, const __grid_constant__ CUtensorMap md) {
  using namespace pcr2;
  using S = Pcr2Shape<N>;
  constexpr int R = S::R, LPS = S::LPS, SPW = S::SPW, TF = S::TF;
  constexpr int BUF = 4 * TF;  // floats per staging buffer (a, b, c, d of a tile)
  constexpr int SYS_STRIDE = S::SYS_STRIDE;
  static_assert(N >= 64 && N <= 1024 && SPW * N == TF, "pcr_twophase: 64 <= n <= 1024");
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
  // this lane's R/4 swizzled 16-byte chunks in a box: chunk index lane*R/4 + q
  int chunk[R / 4];
#pragma unroll
  for (int q = 0; q < R / 4; ++q) {
    const int c = lane * (R / 4) + q, row = c >> 3;
    chunk[q] = row * 32 + (((c & 7) ^ (row & 7)) << 2);
  }
  int k = 0;
  for (long tile = first; tile < tiles; tile += step, ++k) {
    if (!mbar_wait(bar, k & 1, p.status)) break;
    float v[4][R];  // a, b, c, d of the lane's R rows
#pragma unroll
    for (int arr = 0; arr < 4; ++arr)
#pragma unroll
      for (int q = 0; q < R / 4; ++q) {
        const float4 f = *reinterpret_cast<const float4*>(buf + arr * TF + chunk[q]);
        v[arr][4 * q] = f.x; v[arr][4 * q + 1] = f.y; v[arr][4 * q + 2] = f.z; v[arr][4 * q + 3] = f.w;
      }
    // every lane's loads of the buffer are ordered before the bulk copies
    // that refill it with the next tile
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0 && tile + step < tiles) issue(tile + step);
    if (t == 0) v[0][0] = 0.0f;            // a[0] is not part of the system
    if (t == LPS - 1) v[2][R - 1] = 0.0f;  // nor is c[n-1]
    float* sw = scratch + g * SYS_STRIDE;  // this system's transpose scratch (one word array)
    const int rb = t * R;  // this lane's first phase-A row
    const long sys = tile * SPW + g;
    float* dst = gx + sys * N + t;
    if constexpr (PAIRED) {
      NR2 P[R / 2];
#pragma unroll
      for (int j = 0; j < R / 2; ++j) {
        const float2 ib = rcp_approx2(make_float2(v[1][2 * j], v[1][2 * j + 1]));
        P[j] = NR2{__fmul2_rn(make_float2(v[0][2 * j], v[0][2 * j + 1]), ib),
                   __fmul2_rn(make_float2(v[2][2 * j], v[2][2 * j + 1]), ib),
                   __fmul2_rn(make_float2(v[3][2 * j], v[3][2 * j + 1]), ib)};
      }
      phase_a_pairs<LPS, R>(P);
      // ---- transpose, one word array at a time: lane t of system g now
      //      takes rows t + LPS * s ----
      transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].a; });
      transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].c; });
      transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].d; });
      // ---- phase B: distances R .. n/4 ----
      if constexpr (N == 512) {
        NR w[R];
#pragma unroll
        for (int j = 0; j < R / 2; ++j) {
          w[2 * j] = row_x(P[j]);
          w[2 * j + 1] = row_y(P[j]);
        }
        phase_b_xor16<R>(w, lane);
        phase_b_step<1, R>(w);
#pragma unroll
        for (int j = 0; j < R / 2; ++j) P[j] = pair_of(w[2 * j], w[2 * j + 1]);
        phase_b_pairs<2, R>(P);
        phase_b_pairs<4, R>(P);
      } else {
        if constexpr (R <= N / 4) phase_b_pairs<R / LPS, R>(P);
        if constexpr (2 * R <= N / 4) phase_b_pairs<2 * R / LPS, R>(P);
        if constexpr (4 * R <= N / 4) phase_b_pairs<4 * R / LPS, R>(P);
        if constexpr (8 * R <= N / 4) phase_b_pairs<8 * R / LPS, R>(P);
      }
      // ---- 2x2 systems (s, s + R/2), two at a time ----
      if (sys < p.m) {
#pragma unroll
        for (int j = 0; j < R / 4; ++j) {
          const NR2& u = P[j];
          const NR2& l = P[j + R / 4];
          const float2 den = __ffma2_rn(neg2(u.c), l.a, make_float2(1.0f, 1.0f));
          const float2 num = __ffma2_rn(neg2(u.c), l.d, u.d);
          const float2 xu = __fmul2_rn(num, rcp_approx2(den));
          const float2 xl = __ffma2_rn(neg2(l.a), xu, l.d);
          dst[LPS * (2 * j)] = xu.x;
          dst[LPS * (2 * j + 1)] = xu.y;
          dst[LPS * (2 * j + R / 2)] = xl.x;
          dst[LPS * (2 * j + 1 + R / 2)] = xl.y;
        }
      }
    } else {
      NR w[R];
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const float ib = rcp_approx(v[1][q]);
        w[q] = NR{v[0][q] * ib, v[2][q] * ib, v[3][q] * ib};
      }
      phase_a_step<1, LPS, R>(w);
      phase_a_step<2, LPS, R>(w);
      phase_a_step<4, LPS, R>(w);
      phase_a_step<8, LPS, R>(w);
      if constexpr (R >= 32) phase_a_step<16, LPS, R>(w);
      // ---- transpose ----
      {
        NR2 P[R / 2];
#pragma unroll
        for (int j = 0; j < R / 2; ++j) P[j] = pair_of(w[2 * j], w[2 * j + 1]);
        transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].a; });
        transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].c; });
        transpose_word<R, LPS>(sw, rb, t, [&](int j) -> float2& { return P[j].d; });
#pragma unroll
        for (int j = 0; j < R / 2; ++j) {
          w[2 * j] = row_x(P[j]);
          w[2 * j + 1] = row_y(P[j]);
        }
      }
      // ---- phase B ----
      if constexpr (N == 512) {
        phase_b_xor16<R>(w, lane);
        phase_b_step<1, R>(w);
        phase_b_step<2, R>(w);
        phase_b_step<4, R>(w);
      } else {
        if constexpr (R <= N / 4) phase_b_step<R / LPS, R>(w);
        if constexpr (2 * R <= N / 4) phase_b_step<2 * R / LPS, R>(w);
        if constexpr (4 * R <= N / 4) phase_b_step<4 * R / LPS, R>(w);
        if constexpr (8 * R <= N / 4) phase_b_step<8 * R / LPS, R>(w);
      }
      // ---- 2x2 systems (s, s + R/2): x_u + c_u x_l = d_u, a_l x_u + x_l = d_l ----
      if (sys < p.m) {
#pragma unroll
        for (int q = 0; q < R / 2; ++q) {
          const NR& u = w[q];
          const NR& l = w[q + R / 2];
          const float xu = (u.d - u.c * l.d) * rcp_approx(fmaf(-u.c, l.a, 1.0f));
          const float xl = fmaf(-l.a, xu, l.d);
          dst[LPS * q] = xu;
          dst[LPS * (q + R / 2)] = xl;
        }
      }
    }
  }
}

}  // namespace tridi

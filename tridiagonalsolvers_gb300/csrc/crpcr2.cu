// CR-PCR for FP32 systems of 1024 (and, in large batches, 512) unknowns in
// registers, one system a warp (n / 32 contiguous rows a lane, loaded by TMA
// into the warp's buffer): every switch level of "crpcr" (restSystemSize
// 2 .. n/2, crpcr_kernel.cu:1-148, crpcr_app.cu:5) and, at rest 2, "cr"
// (cr_kernel.cu, cr_app.cu:4).
//
// crpcr_lanes_kernel<N, LEV> (rest = N / 2^LEV): the first log2(N/32) CR
// levels run inside the lane (32 -> 16 -> 8 -> 4 -> 2 -> 1 rows at N = 1024; each level's
// last odd row takes its right neighbour from the next lane over one
// shuffle), the levels past five between lanes (lane strides 1, 2, 4, 8).
// PCR on the rows left: distances below the rows a lane holds inside the
// lane, the others between lanes (the neighbour at distance K2 ld is lane
// t -/+ ld, same slot), the closing 2x2 systems between lanes t and t ^ 16.
// The back substitutions retrace the levels from the coefficients each lane
// kept in registers; the lane's 32 unknowns leave in 16-byte stores.  No
// shared memory but the TMA buffer.  At rest 2 the levels and the closing
// solve are CR's own (divisions, unnormalised rows), so cr here rounds
// exactly like every other CR kernel of the library; above rest 2 the
// in-lane levels divide each even row by its diagonal once and eliminate
// against those normalised rows (cr_level_norm).
//
// crpcr512_kernel (rest 512): one CR level inside the lane (on normalised even
// rows, as above) leaves lane t the
// intermediate rows 16t .. 16t+15 as normalised 3-word rows -- exactly the
// 512-row layout of the two-phase PCR (pcr_twophase.cuh, 16 rows a lane, one
// system a warp), so its phase A, transpose, phase B and closing 2x2 systems
// run unchanged and leave x of intermediate row t + 32s in lane t.  Those
// 512 values go through the warp's scratch once (padded so the
// lane-contiguous reads hit distinct banks), each lane forms its 16 even
// rows' x from its own coefficients, and writes its 32 unknowns.  (The lanes
// design at rest 512 -- 16 rows a lane, four PCR steps between lanes with 16
// rows each -- measured 64 % of HBM against this kernel's 80 %, 87 % since
// its level works on normalised even rows.)
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
    // ---- CR level: odd rows 2j+1 against their even neighbours, which are
    //      normalised once (one reciprocal per even row; the back
    //      substitution reuses them) ----
    // (lane 31's last odd row has c = 0, so the shuffled-in neighbour, its
    // own first row, contributes nothing)
    NR e[kRR];  // even row 2j / its diagonal
#pragma unroll
    for (int j = 0; j < kRR; ++j) {
      const float ib = rcp_approx(v[1][2 * j]);
      e[j] = NR{v[0][2 * j] * ib, v[2][2 * j] * ib, v[3][2 * j] * ib};
    }
    const NR eR = shfl_down_nr(e[0], 32);  // the next lane's row 0
    NR2 P[kRR / 2];
#pragma unroll
    for (int j = 0; j < kRR; ++j) {
      const int q = 2 * j + 1;
      const NR& L = e[j];
      const NR& Rn = j + 1 < kRR ? e[j + 1] : eR;
      const float aq = v[0][q], cq = v[2][q];
      const float an = -aq * L.a;
      const float bn = v[1][q] - aq * L.c - cq * Rn.a;
      const float cn = -cq * Rn.c;
      const float dn = v[3][q] - aq * L.d - cq * Rn.d;
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
      xo[q] = e[j].d - e[j].a * xprev - e[j].c * xodd;
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

// The same level with the even rows normalised first, (ea, ec, ed) = (a, c, d)
// / b of row 2j: one reciprocal per even row instead of two per odd row, and
// the back substitution (cr_back_norm) needs none.  The eliminations then
// take the form me - a_q L' - c_q R' with normalised neighbours, which rounds
// differently from CR's own divisions (used where crpcr switches above 2).
template <int K>
__device__ __forceinline__ void cr_level_norm(const float (&a)[K], const float (&b)[K], const float (&c)[K],
                                              const float (&d)[K], float (&ea)[K / 2], float (&ec)[K / 2],
                                              float (&ed)[K / 2], float (&na)[K / 2], float (&nb)[K / 2],
                                              float (&nc)[K / 2], float (&nd)[K / 2]) {
#pragma unroll
  for (int j = 0; j < K / 2; ++j) {
    const float ib = rcp_approx(b[2 * j]);
    ea[j] = a[2 * j] * ib;
    ec[j] = c[2 * j] * ib;
    ed[j] = d[2 * j] * ib;
  }
  const float ra = __shfl_down_sync(kFull, ea[0], 1), rc = __shfl_down_sync(kFull, ec[0], 1);
  const float rd = __shfl_down_sync(kFull, ed[0], 1);
#pragma unroll
  for (int j = 0; j < K / 2; ++j) {
    const int q = 2 * j + 1;
    const float Ra = j + 1 < K / 2 ? ea[j + 1] : ra, Rc = j + 1 < K / 2 ? ec[j + 1] : rc;
    const float Rd = j + 1 < K / 2 ? ed[j + 1] : rd;
    na[j] = -a[q] * ea[j];
    nb[j] = b[q] - a[q] * ec[j] - c[q] * Ra;
    nc[j] = -c[q] * Rc;
    nd[j] = d[q] - a[q] * ed[j] - c[q] * Rd;
  }
}

template <int K>
__device__ __forceinline__ void cr_back_norm(const float (&ea)[K / 2], const float (&ec)[K / 2],
                                             const float (&ed)[K / 2], const float (&xo)[K / 2], float (&x)[K],
                                             int lane) {
  float xprev = __shfl_up_sync(kFull, xo[K / 2 - 1], 1);
  if (lane == 0) xprev = 0.0f;
#pragma unroll
  for (int j = 0; j < K / 2; ++j) {
    x[2 * j] = ed[j] - ea[j] * xprev - ec[j] * xo[j];
    x[2 * j + 1] = xo[j];
    xprev = xo[j];
  }
}

// PCR step between lanes: lane t holds rows K2 t + j, so the neighbours at
// distance K2 ld are lanes t -/+ ld in the same slot.  Lanes whose neighbour
// lies beyond the system's ends receive their own row from the shuffle: the
// coupling there is exactly zero.
template <int K2>
__device__ __forceinline__ void lane_step(NR (&w)[K2], int ld) {
#pragma unroll
  for (int j = 0; j < K2; ++j) {
    const NR L{__shfl_up_sync(kFull, w[j].a, ld), __shfl_up_sync(kFull, w[j].c, ld),
               __shfl_up_sync(kFull, w[j].d, ld)};
    const NR Rr{__shfl_down_sync(kFull, w[j].a, ld), __shfl_down_sync(kFull, w[j].c, ld),
                __shfl_down_sync(kFull, w[j].d, ld)};
    w[j] = step_both(w[j], L, Rr);
  }
}

// PCR on the rows left by the CR levels: lane t holds rows K2 t .. K2 t + K2 - 1
// (unnormalised) of the 32 K2 rows, or, after CR levels between lanes
// (LD0 = 2^levels > 1, K2 = 1), only the lanes t = LD0 j + LD0 - 1 hold a row
// (row j of 32 / LD0).  Distances below K2 run inside the lane, the others
// between lanes (lane distances LD0 .. 8), then the closing 2x2 systems
// pair lane t with lane t ^ 16 in the same slot.  x of the lane's rows out
// (meaningless on lanes that hold no row).
template <int K2, int LD0>
__device__ __forceinline__ void pcr_lanes(const float (&a)[K2], const float (&b)[K2], const float (&c)[K2],
                                          const float (&d)[K2], float (&x)[K2], int lane) {
  NR w[K2];
#pragma unroll
  for (int j = 0; j < K2; ++j) {
    const float ib = rcp_approx(b[j]);
    w[j] = NR{a[j] * ib, c[j] * ib, d[j] * ib};
  }
  if constexpr (K2 >= 2) phase_a_step<1, 32, K2>(w);
  if constexpr (K2 >= 4) phase_a_step<2, 32, K2>(w);
  if constexpr (K2 >= 8) phase_a_step<4, 32, K2>(w);
  if constexpr (K2 >= 16) phase_a_step<8, 32, K2>(w);
#pragma unroll
  for (int ld = LD0; ld < 16; ld *= 2) lane_step<K2>(w, ld);
#pragma unroll
  for (int j = 0; j < K2; ++j) {
    const NR pr = shfl_xor_nr(w[j], 16);
    const NR& u = lane < 16 ? w[j] : pr;  // row r
    const NR& l = lane < 16 ? pr : w[j];  // row r + 16 K2 (r + 16 / LD0 between lanes)
    const float xu = (u.d - u.c * l.d) * rcp_approx(fmaf(-u.c, l.a, 1.0f));
    x[j] = lane < 16 ? xu : fmaf(-l.a, xu, l.d);
  }
}

// L2 CR levels between lanes on a 32-row system held one row a lane (row t in
// lane t), the PCR of the 32 / 2^L2 rows left, and the back substitutions.
// Level i (lane stride s = 2^i) leaves the rows of lanes t with
// (t + 1) mod 2s = 0, each from its neighbours t -/+ s; every lane computes
// (the warp stays converged) and keeps the row it held at each level for the
// back substitution, where the lanes with (t + 1) mod 2s = s take x from
// lanes t -/+ s.  Active rows only ever read active rows; the last row's
// c = 0 zeroes the neighbour that lane 31 receives from itself, and the
// first row's a = 0 the one that lane s - 1 receives from itself.
template <int L2>
__device__ __forceinline__ float cr_cross(float a, float b, float c, float d, int lane) {
  float la[L2], lb[L2], lc[L2], ld[L2];
#pragma unroll
  for (int i = 0; i < L2; ++i) {
    const int s = 1 << i;
    const float aL = __shfl_up_sync(kFull, a, s), bL = __shfl_up_sync(kFull, b, s);
    const float cL = __shfl_up_sync(kFull, c, s), dL = __shfl_up_sync(kFull, d, s);
    const float aR = __shfl_down_sync(kFull, a, s), bR = __shfl_down_sync(kFull, b, s);
    const float cR = __shfl_down_sync(kFull, c, s), dR = __shfl_down_sync(kFull, d, s);
    la[i] = a; lb[i] = b; lc[i] = c; ld[i] = d;
    const float k1 = tdiv(a, bL);
    const float k2 = tdiv(c, bR);
    a = -aL * k1;
    b = b - cL * k1 - aR * k2;
    c = -cR * k2;
    d = d - dL * k1 - dR * k2;
  }
  float x = 0.0f;
  if constexpr (L2 == 4) {
    // two rows left (lanes 15 and 31): CR's closing 2x2 solve on the
    // unnormalised rows, so that cr here rounds like every other CR kernel
    const Row<float> r1{__shfl_sync(kFull, a, 15), __shfl_sync(kFull, b, 15), __shfl_sync(kFull, c, 15),
                        __shfl_sync(kFull, d, 15)};
    const Row<float> r2{__shfl_sync(kFull, a, 31), __shfl_sync(kFull, b, 31), __shfl_sync(kFull, c, 31),
                        __shfl_sync(kFull, d, 31)};
    if (lane == 15) x = solve2_upper(r1, r2);
    if (lane == 31) x = solve2_lower(r1, r2);
  } else {
    const float ta[1] = {a}, tb[1] = {b}, tc[1] = {c}, td[1] = {d};
    float xt[1];
    pcr_lanes<1, (1 << L2)>(ta, tb, tc, td, xt, lane);
    if (((lane + 1) & ((1 << L2) - 1)) == 0) x = xt[0];
  }
#pragma unroll
  for (int i = L2 - 1; i >= 0; --i) {
    const int s = 1 << i;
    const float xL = __shfl_up_sync(kFull, x, s), xR = __shfl_down_sync(kFull, x, s);
    if (((lane + 1) & (2 * s - 1)) == s) x = (ld[i] - la[i] * xL - lc[i] * xR) * rcp_approx(lb[i]);
  }
  return x;
}

// LEV CR levels down from the lane's K rows (the levels past K = 1 between
// lanes), the PCR, and the back substitutions up again.  NORM: the in-lane
// levels on normalised even rows (cr_level_norm); else CR's own arithmetic.
template <int K, int LEV, bool NORM>
__device__ __forceinline__ void cr_solve(const float (&a)[K], const float (&b)[K], const float (&c)[K],
                                         const float (&d)[K], float (&x)[K], int lane) {
  float na[K / 2], nb[K / 2], nc[K / 2], nd[K / 2], xo[K / 2];
  if constexpr (NORM) {
    float ea[K / 2], ec[K / 2], ed[K / 2];
    cr_level_norm<K>(a, b, c, d, ea, ec, ed, na, nb, nc, nd);
    if constexpr (LEV == 1) pcr_lanes<K / 2, 1>(na, nb, nc, nd, xo, lane);
    else if constexpr (K == 2) xo[0] = cr_cross<LEV - 1>(na[0], nb[0], nc[0], nd[0], lane);
    else cr_solve<K / 2, LEV - 1, NORM>(na, nb, nc, nd, xo, lane);
    cr_back_norm<K>(ea, ec, ed, xo, x, lane);
  } else {
    cr_level<K>(a, b, c, d, na, nb, nc, nd);
    if constexpr (LEV == 1) pcr_lanes<K / 2, 1>(na, nb, nc, nd, xo, lane);
    else if constexpr (K == 2) xo[0] = cr_cross<LEV - 1>(na[0], nb[0], nc[0], nd[0], lane);
    else cr_solve<K / 2, LEV - 1, NORM>(na, nb, nc, nd, xo, lane);
    cr_back<K>(a, b, c, d, xo, x, lane);
  }
}

// Shared memory of a lanes-kernel CTA for n unknowns: barriers, then the two
// warps' TMA buffers (1024-byte aligned for the 128-byte swizzle).
constexpr size_t lanes_smem(int n) { return 128 + 1024 + (size_t)kWarps * 4 * n * 4; }

// CR-PCR with the switch at N / 2^LEV for N = 512 or 1024 unknowns (R = N / 32
// rows a lane), in registers and shuffles (the file header gives the scheme).
// At 1024 unknowns four CTAs of two warps an SM (at most 255 registers: none
// spill; three or five to six measured the same or slower), at 512 eight (the
// same bytes of tiles in flight an SM).
template <int N, int LEV>
__global__ void __launch_bounds__(kWarps * 32, N == 512 ? 8 : 4)
    crpcr_lanes_kernel(HybridParams p, const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                       const __grid_constant__ CUtensorMap mc, const __grid_constant__ CUtensorMap md) {
  constexpr int R = N / 32, TF = N;
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + warp;
  const uint32_t base = smem_addr(smem);
  const uint32_t ring = (base + 128 + 1023) & ~1023u;
  float* buf = reinterpret_cast<float*>(smem + (ring - base)) + (size_t)warp * 4 * TF;
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
    const int row = (int)(tile * (TF / 32));
    mbar_arrive_expect_tx(bar, 4 * TF * sizeof(float));
    tma_load_2d(buf + 0 * TF, &ma, 0, row, bar);
    tma_load_2d(buf + 1 * TF, &mb, 0, row, bar);
    tma_load_2d(buf + 2 * TF, &mc, 0, row, bar);
    tma_load_2d(buf + 3 * TF, &md, 0, row, bar);
  };
  if (lane == 0 && first < tiles) issue(first);
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
    if (lane == 0) v[0][0] = 0.0f;
    if (lane == 31) v[2][R - 1] = 0.0f;
    float x[R];
    // rest 2 is cr: CR's own arithmetic, bit for bit that of the other CR kernels
    cr_solve<R, LEV, ((N >> LEV) > 2)>(v[0], v[1], v[2], v[3], x, lane);
    float4* dst = reinterpret_cast<float4*>(gx + tile * N + R * lane);
#pragma unroll
    for (int q = 0; q < R / 4; ++q) dst[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
  }
}

using TileKernel = void (*)(HybridParams, CUtensorMap, CUtensorMap, CUtensorMap, CUtensorMap);

// One warp a system, as many CTAs of two warps as fit on every SM up to
// max_per_sm (the warps then loop over the batch).  At 1024 unknowns five or
// six CTAs an SM, where the registers allow it, measured 5 % slower than four:
// more warps contend for the shared-memory pipe without hiding more DRAM
// latency.
tridi_status launch_tiles(TileKernel kern, size_t smem, int max_per_sm, const HybridParams& p,
                          const CUtensorMap* tm, const DeviceInfo* dev, cudaStream_t stream) {
  if (smem > (size_t)dev->max_smem_optin) return TRIDI_ERROR_UNSUPPORTED_SIZE;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
  if (e != cudaSuccess) return cuda_status(e);
  if (per_sm < 1) per_sm = 1;
  if (per_sm > max_per_sm) per_sm = max_per_sm;
  long grid = (long)per_sm * dev->sm_count;
  if (grid * kWarps > p.m) grid = (p.m + kWarps - 1) / kWarps;
  kern<<<(unsigned)grid, kWarps * 32, smem, stream>>>(p, tm[0], tm[1], tm[2], tm[3]);
  return cuda_status(cudaGetLastError());
}

template <int N>
tridi_status launch_lanes(int stride, const HybridParams& p, const CUtensorMap* tm, const DeviceInfo* dev,
                          cudaStream_t stream) {
  constexpr int M = N == 512 ? 8 : 4;
  constexpr size_t S = lanes_smem(N);
  switch (stride) {
    case 2: if constexpr (N == 512) return launch_tiles(crpcr_lanes_kernel<N, 1>, S, M, p, tm, dev, stream);
            break;
    case 4: return launch_tiles(crpcr_lanes_kernel<N, 2>, S, M, p, tm, dev, stream);
    case 8: return launch_tiles(crpcr_lanes_kernel<N, 3>, S, M, p, tm, dev, stream);
    case 16: return launch_tiles(crpcr_lanes_kernel<N, 4>, S, M, p, tm, dev, stream);
    case 32: return launch_tiles(crpcr_lanes_kernel<N, 5>, S, M, p, tm, dev, stream);
    case 64: return launch_tiles(crpcr_lanes_kernel<N, 6>, S, M, p, tm, dev, stream);
    case 128: return launch_tiles(crpcr_lanes_kernel<N, 7>, S, M, p, tm, dev, stream);
    case 256: return launch_tiles(crpcr_lanes_kernel<N, 8>, S, M, p, tm, dev, stream);
    case 512: if constexpr (N == 1024) return launch_tiles(crpcr_lanes_kernel<N, 9>, S, M, p, tm, dev, stream);
              break;
    default: break;
  }
  return TRIDI_ERROR_UNSUPPORTED_SIZE;
}

}  // namespace

// True when a register kernel takes this FP32 call: cr, or crpcr at any
// switch level (stride = n / rest = 2 .. n/2), at n = 1024, or at n = 512 from
// 4096 systems up (on a small batch one warp a system leaves the GPU short of
// threads: 512 x 512 cr 6.1 us against 4.7 us for the block kernel, which
// gives a system two warps; 32768 x 512 cr 54.6 against 58.0 us, crpcr rest
// 256 55.9 against 117.2 us), 16-byte aligned a..d and x, the batch within
// the tensor maps' 32-bit row count.
bool crpcr_regs_applies(const void* a, const void* b, const void* c, const void* d, const void* x, int n, long m,
                        int stride) {
  return (n == 1024 || (n == 512 && m >= 4096)) && stride >= 2 && stride <= n / 2 && is_pow2(stride) &&
         aligned16(a) &&
         aligned16(b) && aligned16(c) && aligned16(d) && aligned16(x) && m * n / 32 < (1L << 31) &&
         tunable(TRIDI_TUNE_PCR_KERNEL) != 2 && !g_host_mapped_io;
}

tridi_status crpcr_regs_solve(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                              int m, int stride, cudaStream_t stream) {
  const DeviceInfo* dev = current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  HybridParams p{};
  p.a = a; p.b = b; p.c = c; p.d = d; p.x = x;
  p.n = n; p.m = m; p.stride = stride;
  p.status = dev->status;
  const uint64_t rows = (uint64_t)m * n / 32;
  const uint32_t box = (uint32_t)(n / 32);  // a system: n / 32 rows of 32 values
  CUtensorMap tma, tmb, tmc, tmd;
  if (!make_tensor_map_2d(&tma, a, 32, rows, 128, 32, box, true) ||
      !make_tensor_map_2d(&tmb, b, 32, rows, 128, 32, box, true) ||
      !make_tensor_map_2d(&tmc, c, 32, rows, 128, 32, box, true) ||
      !make_tensor_map_2d(&tmd, d, 32, rows, 128, 32, box, true))
    return cuda_status(cudaErrorInvalidValue);
  const CUtensorMap tm[4] = {tma, tmb, tmc, tmd};
  if (n == 512) return launch_lanes<512>(stride, p, tm, dev, stream);
  if (stride == 2) return launch_tiles(crpcr512_kernel, kSmem, 4, p, tm, dev, stream);
  return launch_lanes<1024>(stride, p, tm, dev, stream);
}

}  // namespace tridi

// The cyclic-reduction family on sm_103a: CR, PCR and the hybrid CR -> PCR ->
// CR with a tunable switch level, all as one kernel template.
//
// Algorithm (the reference's, unchanged in its arithmetic):
//   * CR forward levels s = 2, 4, ..., stride eliminate every row i with
//     i % s == s-1 against rows i -/+ s/2 (right neighbour clamped to n-1),
//     crpcr_kernel.cu:40-59.
//   * The remaining rest = n/stride rows (i % stride == stride-1) form the
//     intermediate system.  log2(rest/2) PCR steps with delta = 1, 2, ...,
//     rest/4 leave rest/2 independent 2x2 systems (j, j + rest/2),
//     crpcr_kernel.cu:81-119 (which clamps the neighbours outside the system
//     to the first / last row; the shuffle paths here use identity rows,
//     the same values for a[0] = c[n-1] = 0).
//   * CR back substitution for levels s = stride, ..., 2, crpcr_kernel.cu:127-141.
//   stride = n/2 is plain CR (cr_kernel.cu), stride = 1 is plain PCR
//   (pcr_kernel.cu), anything between is crpcr with rest = n/stride.
//
// Mapping to the GB300 (not the reference's one-thread-per-pair layout):
//   * A system is owned by a group of TPS = n/K threads; thread t holds rows
//     [tK, tK+K) in registers.  The first log2(K) CR levels run inside each
//     thread; only the thread's last row needs data from the next thread
//     (one shuffle per level).
//   * The cross-thread levels, the PCR steps and the 2x2 solves run on warp
//     shuffles when the group fits in a warp (TPS <= 32) and on shared memory
//     with named barriers otherwise.
//   * Input rows arrive through a persistent pipeline: one producer warp
//     streams whole tiles (G consecutive systems of a, b, c, d) into an
//     S-stage shared-memory ring with cp.async.bulk + mbarrier transaction
//     counts; the consumer warps read their rows with 16-byte shared loads,
//     release the stage, solve, and write x with 16-byte global stores.
//     Inputs too small or misaligned for bulk copies are read directly.
#pragma once
#include <type_traits>

#include "tridi_device.cuh"

namespace tridi {

struct HybridParams {
  const void* a;
  const void* b;
  const void* c;
  const void* d;
  void* x;
  int n;         // system size (power of two)
  int m;         // number of systems
  int tps;       // threads per system, n / K
  int G;         // systems per tile
  int ntiles;    // ceil(m / G)
  int stride;    // n / rest: 1 = PCR, n/2 = CR
  int stages;    // pipeline depth (0 = direct loads, no bulk copies)
  int ct;        // consumer threads per CTA = G * tps
  int scratch_rows;  // rows of the block-path scratch per group
  unsigned* status;
};

template <int V>
struct Log2 {
  static constexpr int value = 1 + Log2<V / 2>::value;
};
template <>
struct Log2<1> {
  static constexpr int value = 0;
};

// Shared-memory scratch used by the block (TPS > 32) path; laid out after the
// pipeline stages.  Per group: 4 arrays of `rows` entries plus x.
template <class T>
struct GroupScratch {
  T* a;
  T* b;
  T* c;
  T* d;
  T* x;
  __device__ Row<T> get(int i) const { return {a[i], b[i], c[i], d[i]}; }
  __device__ void put(int i, const Row<T>& r) const {
    a[i] = r.a; b[i] = r.b; c[i] = r.c; d[i] = r.d;
  }
};

// ---------------------------------------------------------------------------
// In-thread CR levels s = 2 .. SMAX (SMAX <= K), every row but the thread's
// last (whose right neighbour lives in the next thread).
template <class T, int K, int SMAX>
__device__ __forceinline__ void local_forward(Row<T> (&r)[K]) {
  constexpr int LOGK = Log2<K>::value;
#pragma unroll
  for (int j = 0; j < LOGK; ++j) {
    const int s = 2 << j;
    if (s <= SMAX) {
#pragma unroll
      for (int i = s - 1; i < K - 1; i += s) r[i] = reduce_row(r[i], r[i - s / 2], r[i + s / 2]);
    }
  }
}

// In-thread CR back substitution for levels s = SMAX .. 2.
// xr[i] must already hold x for every row with i % (2*smax) == 2*smax-1
// handled by coarser levels; x_prev is x of the previous thread's last row.
template <class T, int K, int SMAX>
__device__ __forceinline__ void local_backward(const Row<T> (&r)[K], T (&xr)[K], T x_prev, bool first_thread) {
  constexpr int LOGK = Log2<K>::value;
#pragma unroll
  for (int j = LOGK - 1; j >= 0; --j) {
    const int s = 2 << j;
    if (s <= SMAX) {
#pragma unroll
      for (int i = s / 2 - 1; i < K; i += s) {
        const bool edge = (i == s / 2 - 1);
        const T xl = edge ? x_prev : xr[i >= s / 2 ? i - s / 2 : 0];
        xr[i] = back_row(r[i], xl, xr[i + s / 2], edge && first_thread);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// PCR on the intermediate system when it has R = K/STRIDE rows per thread
// (local rows STRIDE*q + STRIDE-1), warp-shuffle version (TPS <= 32).
// Leaves x of those rows in xr.
template <class T, int K, int STRIDE>
__device__ __forceinline__ void pcr_regs_warp(const Row<T> (&r)[K], T (&xr)[K], int t, int tps) {
  constexpr int R = K / STRIDE;
  constexpr int LOGMAX = Log2<R>::value + 5;  // rest <= 32 * R
  Row<T> y[R];
#pragma unroll
  for (int q = 0; q < R; ++q) y[q] = r[STRIDE * q + STRIDE - 1];
  const int rest = tps * R;
  // The system's ends couple to nothing outside it (the gold solver's
  // a[0] = c[n-1] = 0).  With those two couplings exactly zero, a row whose
  // neighbour at distance dl lies outside the system has an exactly zero
  // coupling to it at step dl (by induction over the steps), so any finite
  // row whose b is a pivot can stand in for the outside one: the shuffles
  // below hand an out-of-range lane its own row and need no selects.  The
  // reference clamps to the first / last row instead (pcr_kernel.cu:33-37):
  // the same values.
  if (t == 0) y[0].a = T(0);
  if (t == tps - 1) y[R - 1].c = T(0);
  // Every row is the divisor of its two neighbours at each step: its owner
  // divides it by its diagonal once and hands (a/b, c/b, d/b) to them
  // (reduce_row_nrm): one reciprocal per row and step instead of two, three
  // shuffled values per neighbour instead of four.
#pragma unroll
  for (int e = 0; e < LOGMAX; ++e) {
    const int dl = 1 << e;
    if (4 * dl <= rest) {  // delta = 1 .. rest/4
      NRow<T> w[R];
#pragma unroll
      for (int q = 0; q < R; ++q) w[q] = normalize_row(y[q]);
      Row<T> ny[R];
      if (dl < R) {
        NRow<T> fromL[R], fromR[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
          if (q < dl) fromL[q] = shfl_up(w[(R - dl + q) % R], 1, tps);
          if (q < dl) fromR[q] = shfl_down(w[q % R], 1, tps);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const NRow<T> L = q >= dl ? w[(q - dl + R) % R] : fromL[q];
          const NRow<T> Rr = q + dl < R ? w[(q + dl) % R] : fromR[(q + dl - R + R) % R];
          ny[q] = reduce_row_nrm(y[q], L, Rr);
        }
      } else {
        const int ex = dl / R;  // whole threads away
#pragma unroll
        for (int q = 0; q < R; ++q)
          ny[q] = reduce_row_nrm(y[q], shfl_up(w[q], ex, tps), shfl_down(w[q], ex, tps));
      }
#pragma unroll
      for (int q = 0; q < R; ++q) y[q] = ny[q];
    }
  }
  // 2x2 systems (j, j + rest/2): same local slot, thread t ^ tps/2.  Each
  // side needs the partner's d/b and its coupling to this side over b (c/b
  // from the upper row, a/b from the lower): x = (d - k d') / (b - k k'),
  // k this row's coupling to the partner.
  const bool upper = t < tps / 2;
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const NRow<T> w = normalize_row(y[q]);
    const T pd = __shfl_xor_sync(kFull, w.d, tps / 2, tps);
    const T pk = __shfl_xor_sync(kFull, upper ? w.c : w.a, tps / 2, tps);
    const T k = upper ? y[q].c : y[q].a;
    xr[STRIDE * q + STRIDE - 1] = tdiv(y[q].d - k * pd, y[q].b - k * pk);
  }
}

// Same, shared-memory version for groups wider than a warp.
template <class T, int K, int STRIDE>
__device__ __forceinline__ void pcr_regs_block(const Row<T> (&r)[K], T (&xr)[K], int t, int tps,
                                               const GroupScratch<T>& sc, int ct) {
  constexpr int R = K / STRIDE;
  // Row j of the intermediate system (thread j / R, slot j % R) is kept at
  // scratch index (j % R) * tps + j / R: at a fixed slot the threads of a
  // warp touch consecutive words, whatever the PCR distance.
  auto at = [tps](int j) { return (j % R) * tps + j / R; };
  Row<T> y[R];
#pragma unroll
  for (int q = 0; q < R; ++q) y[q] = r[STRIDE * q + STRIDE - 1];
  // end couplings zeroed, normalised rows exchanged: as in pcr_regs_warp
  // (the clamped neighbours of the rows near the ends then contribute
  // exactly nothing; three words per row in shared memory instead of four)
  if (t == 0) y[0].a = T(0);
  if (t == tps - 1) y[R - 1].c = T(0);
  const int rest = tps * R;
  for (int dl = 1; 4 * dl <= rest; dl *= 2) {
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const NRow<T> w = normalize_row(y[q]);
      sc.a[q * tps + t] = w.a;
      sc.c[q * tps + t] = w.c;
      sc.d[q * tps + t] = w.d;
    }
    consumer_sync(ct);
    Row<T> ny[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int j = t * R + q;
      const int ol = at(j - dl < 0 ? 0 : j - dl);
      const int orr = at(j + dl > rest - 1 ? rest - 1 : j + dl);
      ny[q] = reduce_row_nrm(y[q], NRow<T>{sc.a[ol], sc.c[ol], sc.d[ol]}, NRow<T>{sc.a[orr], sc.c[orr], sc.d[orr]});
    }
    consumer_sync(ct);
#pragma unroll
    for (int q = 0; q < R; ++q) y[q] = ny[q];
  }
  // 2x2 systems (j, j + rest/2): x = (d - k d') / (b - k k') with the
  // partner's normalised d and coupling to this row (see pcr_regs_warp)
  const int half = rest / 2;
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int j = t * R + q;
    const NRow<T> w = normalize_row(y[q]);
    sc.a[q * tps + t] = j < half ? w.c : w.a;
    sc.d[q * tps + t] = w.d;
  }
  consumer_sync(ct);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int j = t * R + q;
    const int o = at(j < half ? j + half : j - half);
    const T k = j < half ? y[q].c : y[q].a;
    xr[STRIDE * q + STRIDE - 1] = tdiv(y[q].d - k * sc.d[o], y[q].b - k * sc.a[o]);
  }
}

// ---------------------------------------------------------------------------
// Whole-system solve for one group.  r: the thread's K rows (consumed), xr:
// the thread's K unknowns (out).  LSTRIDE = 0 when the intermediate system
// has at most one row per thread (stride >= K), else LSTRIDE = stride < K.
template <class T, int K, bool WARP, int LSTRIDE>
__device__ __forceinline__ void hybrid_solve(Row<T> (&r)[K], T (&xr)[K], int t, int tps, int stride,
                                             const GroupScratch<T>& sc, Row<T>* exports, int ct) {
  constexpr int LOGK = Log2<K>::value;
  constexpr int SMAX = LSTRIDE == 0 ? K : LSTRIDE;  // last in-thread CR level
  const bool last_thread = (t == tps - 1);
  const int lane = threadIdx.x & 31;

  // 1. In-thread CR levels for every row but the last.
  local_forward<T, K, SMAX>(r);

  // 2. The last row's CR levels: its right neighbour at level s is the next
  //    thread's row s/2-1, already final after step 1.
  if constexpr (!WARP) {
    if (LOGK > 0 && lane == 0) {
#pragma unroll
      for (int j = 0; j < LOGK; ++j) exports[(threadIdx.x >> 5) * LOGK + j] = r[(1 << j) - 1];
    }
    consumer_sync(ct);
  }
#pragma unroll
  for (int j = 0; j < LOGK; ++j) {
    const int s = 2 << j;
    if (s <= SMAX) {
      Row<T> R = shfl_down(r[(1 << j) - 1], 1, WARP ? tps : 32);
      if constexpr (!WARP) {
        if (lane == 31 && !last_thread) R = exports[((threadIdx.x >> 5) + 1) * LOGK + j];
      }
      if (last_thread) R = r[K - 1];
      r[K - 1] = reduce_row(r[K - 1], r[K - 1 - s / 2], R);
    }
  }

  T x_prev;
  if constexpr (LSTRIDE == 0) {
    // 3a. One row per thread remains (row tK+K-1).  Cross-thread CR levels
    //     until the intermediate system is reached (threads spaced P apart),
    //     then PCR on it and the 2x2 solves, then CR back substitution.
    Row<T> C = r[K - 1];
    const int P = stride / K;
    const int rest = tps / P;
    const bool on = ((t + 1) & (P - 1)) == 0;
    const int j = (t + 1) / P - 1;
    T xC = T(0);
    if constexpr (WARP) {
      // Levels unrolled to their bound (tps <= 32: P <= 16, rest <= 32, so
      // at most 4 of each) under warp-uniform conditions; every lane
      // computes each step and the lanes the step is for keep the result
      // (selects, no divergent branches).
      constexpr int kLevels = 4;
      // (the last thread's right neighbour is clamped to itself, as in
      // cr_kernel.cu:52: shfl_down hands an out-of-range lane its own row)
#pragma unroll
      for (int e = 0; e < kLevels; ++e) {
        const int D = 1 << e;
        if (D < P) {
          const Row<T> L = shfl_up(C, D, tps);
          const Row<T> R = shfl_down(C, D, tps);
          const Row<T> N = reduce_row(C, L, R);
          if (((t + 1) & (2 * D - 1)) == 0) C = N;
        }
      }
      // PCR with the system's end couplings zeroed: out-of-range lanes get
      // their own row, which contributes nothing (see pcr_regs_warp)
      if (on && j == 0) C.a = T(0);
      if (on && j == rest - 1) C.c = T(0);
#pragma unroll
      for (int e = 0; e < kLevels; ++e) {
        const int dl = 1 << e;
        if (4 * dl <= rest) {
          const int dd = dl * P;
          const Row<T> L = shfl_up(C, dd, tps);
          const Row<T> R = shfl_down(C, dd, tps);
          const Row<T> N = reduce_row(C, L, R);
          if (on) C = N;
        }
      }
      const Row<T> pr = shfl_xor(C, tps / 2, tps);
      if (on) xC = (t < tps / 2) ? solve2_upper(C, pr) : solve2_lower(pr, C);
#pragma unroll
      for (int e = kLevels - 1; e >= 0; --e) {
        const int D = 1 << e;
        if (D < P) {
          const T xl = __shfl_up_sync(kFull, xC, D, tps);
          const T xrr = __shfl_down_sync(kFull, xC, D, tps);
          const T v = back_row(C, xl, xrr, t == D - 1);
          if (((t + 1) & (2 * D - 1)) == D) xC = v;
        }
      }
      x_prev = __shfl_up_sync(kFull, xC, 1, tps);
    } else if (P >= 32) {
      // Block group, levels D = 1..16 inside each warp on shuffles.  Lane 31's
      // right neighbour at level D is the next warp's lane D-1, final after
      // level D/2: lane 31 first runs these levels with its own row in that
      // place, then redoes them once the next warp has exported those rows
      // (no other lane reads lane 31's rows below level 32: the neighbours
      // of lane l at level D are lanes l -/+ D <= 30).  The same operands
      // reach every reduce_row as in the shared-memory form below.
      const int lane = threadIdx.x & 31, wcta = threadIdx.x >> 5;
      Row<T>* ex2 = exports + (ct / 32 + 1) * (LOGK > 0 ? LOGK : 1);
      const Row<T> c0 = C;
      Row<T> left[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        const int D = 1 << e;
        left[e] = shfl_up(C, D, 32);
        const Row<T> N = reduce_row(C, left[e], shfl_down(C, D, 32));
        if (((lane + 1) & (2 * D - 1)) == 0) C = N;
      }
      if (lane < 16 && (lane & (lane + 1)) == 0) ex2[wcta * 5 + (31 - __clz(lane + 1))] = C;
      consumer_sync(ct);
      if (lane == 31 && !last_thread) {
        Row<T> c = c0;
#pragma unroll
        for (int e = 0; e < 5; ++e) c = reduce_row(c, left[e], ex2[(wcta + 1) * 5 + e]);
        C = c;
      }
      sc.put(t, C);
      consumer_sync(ct);
      for (int D = 32; D < P; D *= 2) {  // across warps
        if (((t + 1) & (2 * D - 1)) == 0) {
          const int tr = t + D > tps - 1 ? tps - 1 : t + D;
          C = reduce_row(C, sc.get(t - D), sc.get(tr));
          sc.put(t, C);
        }
        consumer_sync(ct);
      }
      for (int dl = 1; 4 * dl <= rest; dl *= 2) {
        Row<T> nc = C;
        if (on) {
          const int jl = j - dl < 0 ? 0 : j - dl;
          const int jr = j + dl > rest - 1 ? rest - 1 : j + dl;
          nc = reduce_row(C, sc.get((jl + 1) * P - 1), sc.get((jr + 1) * P - 1));
        }
        consumer_sync(ct);
        if (on) {
          C = nc;
          sc.put(t, C);
        }
        consumer_sync(ct);
      }
      if (on) {
        const int pt = t ^ (tps / 2);
        xC = (t < tps / 2) ? solve2_upper(C, sc.get(pt)) : solve2_lower(sc.get(pt), C);
        sc.x[t] = xC;
      }
      consumer_sync(ct);
      for (int D = P / 2; D >= 32; D /= 2) {
        if (((t + 1) & (2 * D - 1)) == D) {
          const T xl = (t - D >= 0) ? sc.x[t - D] : T(0);
          xC = back_row(C, xl, sc.x[t + D], t == D - 1);
          sc.x[t] = xC;
        }
        consumer_sync(ct);
      }
      // levels D = 16..1 inside each warp; lane D-1's left neighbour is the
      // previous warp's lane 31, whose x is in sc.x
      const T xpw = (t - lane > 0) ? sc.x[t - lane - 1] : T(0);
#pragma unroll
      for (int e = 4; e >= 0; --e) {
        const int D = 1 << e;
        const T xu = __shfl_up_sync(kFull, xC, D, 32);
        const T xrr = __shfl_down_sync(kFull, xC, D, 32);
        const T v = back_row(C, lane < D ? xpw : xu, xrr, t == D - 1);
        if (((lane + 1) & (2 * D - 1)) == D) xC = v;
      }
      const T xu = __shfl_up_sync(kFull, xC, 1, 32);
      x_prev = lane == 0 ? xpw : xu;
    } else if (rest <= 64) {
      // Block group, P < 32: the CR levels D < P stay inside each warp (as
      // above, lane 31 redoes its chain from the next warp's exported rows);
      // the rest <= 64 rows of the intermediate system are gathered into the
      // group's first warp (1 or 2 consecutive rows a lane), which solves
      // them with pcr_regs_warp (PCR on shuffles and the closing 2x2
      // systems), with no barrier in between; the back substitution is in
      // each warp again.
      const int lane = threadIdx.x & 31, wcta = threadIdx.x >> 5;
      Row<T>* ex2 = exports + (ct / 32 + 1) * (LOGK > 0 ? LOGK : 1);
      const Row<T> c0 = C;
      Row<T> left[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int D = 1 << e;
        if (D < P) {
          left[e] = shfl_up(C, D, 32);
          const Row<T> N = reduce_row(C, left[e], shfl_down(C, D, 32));
          if (((lane + 1) & (2 * D - 1)) == 0) C = N;
        }
      }
      if (lane < 16 && (lane & (lane + 1)) == 0 && lane + 1 < P) ex2[wcta * 5 + (31 - __clz(lane + 1))] = C;
      consumer_sync(ct);
      if (lane == 31 && !last_thread) {
        Row<T> c = c0;
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if ((1 << e) < P) c = reduce_row(c, left[e], ex2[(wcta + 1) * 5 + e]);
        C = c;
      }
      if (on) sc.put(j, C);
      consumer_sync(ct);
      if ((t >> 5) == 0) {  // the group's first warp
        const auto solve_gathered = [&](auto rows_tag) {
          constexpr int RL = decltype(rows_tag)::value;  // intermediate rows a lane
          const int lanes = rest / RL;                    // lanes holding them (a power of two <= 32)
          Row<T> y[RL];
          T xs[RL];
#pragma unroll
          for (int q = 0; q < RL; ++q)
            y[q] = lane < lanes ? sc.get(lane * RL + q) : Row<T>{T(0), T(1), T(0), T(0)};
          pcr_regs_warp<T, RL, 1>(y, xs, lane & (lanes - 1), lanes);
          if (lane < lanes) {
#pragma unroll
            for (int q = 0; q < RL; ++q) sc.x[lane * RL + q] = xs[q];
          }
        };
        if (rest <= 32)
          solve_gathered(std::integral_constant<int, 1>{});
        else
          solve_gathered(std::integral_constant<int, 2>{});
      }
      consumer_sync(ct);
      if (on) xC = sc.x[j];
      // back substitution D = P/2..1 inside each warp; lane D-1's left
      // neighbour is the previous warp's lane 31 (intermediate row
      // 32 w / P - 1)
      const int w0 = t - lane;  // the warp's first thread in the group
      const T xpw = w0 > 0 ? sc.x[w0 / P - 1] : T(0);
#pragma unroll
      for (int e = 3; e >= 0; --e) {
        const int D = 1 << e;
        if (D < P) {
          const T xu = __shfl_up_sync(kFull, xC, D, 32);
          const T xrr = __shfl_down_sync(kFull, xC, D, 32);
          const T v = back_row(C, lane < D ? xpw : xu, xrr, t == D - 1);
          if (((lane + 1) & (2 * D - 1)) == D) xC = v;
        }
      }
      const T xu = __shfl_up_sync(kFull, xC, 1, 32);
      x_prev = lane == 0 ? xpw : xu;
    } else {
      sc.put(t, C);
      consumer_sync(ct);
      for (int D = 1; D < P; D *= 2) {
        if (((t + 1) & (2 * D - 1)) == 0) {
          const int tr = t + D > tps - 1 ? tps - 1 : t + D;
          C = reduce_row(C, sc.get(t - D), sc.get(tr));
          sc.put(t, C);
        }
        consumer_sync(ct);
      }
      for (int dl = 1; 4 * dl <= rest; dl *= 2) {
        Row<T> nc = C;
        if (on) {
          const int jl = j - dl < 0 ? 0 : j - dl;
          const int jr = j + dl > rest - 1 ? rest - 1 : j + dl;
          nc = reduce_row(C, sc.get((jl + 1) * P - 1), sc.get((jr + 1) * P - 1));
        }
        consumer_sync(ct);
        if (on) {
          C = nc;
          sc.put(t, C);
        }
        consumer_sync(ct);
      }
      if (on) {
        const int pt = t ^ (tps / 2);
        xC = (t < tps / 2) ? solve2_upper(C, sc.get(pt)) : solve2_lower(sc.get(pt), C);
        sc.x[t] = xC;
      }
      consumer_sync(ct);
      for (int D = P / 2; D >= 1; D /= 2) {
        if (((t + 1) & (2 * D - 1)) == D) {
          const T xl = (t - D >= 0) ? sc.x[t - D] : T(0);
          xC = back_row(C, xl, sc.x[t + D], t == D - 1);
          sc.x[t] = xC;
        }
        consumer_sync(ct);
      }
      x_prev = (t > 0) ? sc.x[t - 1] : T(0);
    }
    xr[K - 1] = xC;
  } else {
    // 3b. The intermediate system has K/stride rows in every thread: PCR.
    if constexpr (WARP) pcr_regs_warp<T, K, LSTRIDE>(r, xr, t, tps);
    else pcr_regs_block<T, K, LSTRIDE>(r, xr, t, tps, sc, ct);
    if constexpr (WARP) {
      x_prev = __shfl_up_sync(kFull, xr[K - 1], 1, tps);
    } else {
      consumer_sync(ct);  // sc reused for x below
      sc.x[t] = xr[K - 1];
      consumer_sync(ct);
      x_prev = (t > 0) ? sc.x[t - 1] : T(0);
    }
  }

  // 4. In-thread CR back substitution.
  local_backward<T, K, SMAX>(r, xr, x_prev, t == 0);
}

// ---------------------------------------------------------------------------
// Shared-memory layout helpers (host and device agree on these).
template <class T>
struct HybridSmem {
  // [full[S] | empty[S]] barriers (128 B), S stages of 4*G*n T, then the
  // block-path scratch: G groups * 5 * rows T, then exports (per warp: its
  // lane 0's rows of the in-thread levels, then 5 rows of the in-warp levels).
  static __host__ __device__ size_t barrier_bytes() { return 128; }
  static __host__ __device__ size_t stage_elems(int G, int n) { return (size_t)4 * G * n; }
  static __host__ __device__ size_t bytes(int stages, int G, int n, int rows, bool warp, int ct, int logk) {
    size_t s = barrier_bytes() + (size_t)stages * stage_elems(G, n) * sizeof(T);
    if (!warp) {
      s += (size_t)G * 5 * rows * sizeof(T);
      s += (size_t)(ct / 32 + 1) * ((logk > 0 ? logk : 1) + 5) * sizeof(Row<T>);
    }
    return s;
  }
};

constexpr int kWarpKernelThreads = 128;  // hybrid_warp_kernel: 4 warps per CTA

template <class T, int K, bool WARP, int LSTRIDE, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) hybrid_kernel(HybridParams p) {
  constexpr int LOGK = Log2<K>::value;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + 8;
  const int S = p.stages;
  const int n = p.n, G = p.G, tps = p.tps, ct = p.ct;
  T* stages = reinterpret_cast<T*>(smem + HybridSmem<T>::barrier_bytes());
  const size_t stage_elems = HybridSmem<T>::stage_elems(G, n);

  const int tid = threadIdx.x;
  const bool producer = tid >= ct;

  if (tid == 0 && S > 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], ct / 32);
    }
    mbar_fence_init();
  }
  __syncthreads();

  const T* ga = static_cast<const T*>(p.a);
  const T* gb = static_cast<const T*>(p.b);
  const T* gc = static_cast<const T*>(p.c);
  const T* gd = static_cast<const T*>(p.d);
  T* gx = static_cast<T*>(p.x);

  if (producer) {
    // ---- producer warp: lane 0 streams tiles into the ring ----
    if (S > 0 && (tid & 31) == 0) {
      int k = 0;
      for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
        const int s = k % S;
        if (k >= S && !mbar_wait(&empty[s], ((k / S) - 1) & 1, p.status)) break;
        const long sys0 = (long)tile * G;
        const long nsys = (p.m - sys0) < G ? (p.m - sys0) : G;
        const uint32_t bytes = (uint32_t)(nsys * n * sizeof(T));
        T* st = stages + s * stage_elems;
        mbar_arrive_expect_tx(&full[s], 4 * bytes);
        bulk_g2s(st + 0 * (size_t)G * n, ga + sys0 * n, bytes, &full[s]);
        bulk_g2s(st + 1 * (size_t)G * n, gb + sys0 * n, bytes, &full[s]);
        bulk_g2s(st + 2 * (size_t)G * n, gc + sys0 * n, bytes, &full[s]);
        bulk_g2s(st + 3 * (size_t)G * n, gd + sys0 * n, bytes, &full[s]);
      }
    }
    return;
  }

  // ---- consumer warps ----
  const int g = tid / tps;
  const int t = tid - g * tps;
  GroupScratch<T> sc{};
  Row<T>* exports = nullptr;
  if constexpr (!WARP) {
    T* base = stages + (size_t)S * stage_elems;
    const size_t rows = p.scratch_rows;
    T* mine = base + (size_t)g * 5 * rows;
    sc = GroupScratch<T>{mine, mine + rows, mine + 2 * rows, mine + 3 * rows, mine + 4 * rows};
    exports = reinterpret_cast<Row<T>*>(base + (size_t)G * 5 * rows);
  }

  int k = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
    const long sys = (long)tile * G + g;
    Row<T> r[K];
    T va[K], vb[K], vc[K], vd[K];
    bool ok = true;
    if (S > 0) {
      const int s = k % S;
      ok = mbar_wait(&full[s], (k / S) & 1, p.status);
      if constexpr (!WARP) ok = consumer_sync_and(ct, ok);
      if (!ok) break;
      const T* st = stages + s * stage_elems + (size_t)g * n + (size_t)t * K;
      load_vec_smem<T, K>(st + 0 * (size_t)G * n, va);
      load_vec_smem<T, K>(st + 1 * (size_t)G * n, vb);
      load_vec_smem<T, K>(st + 2 * (size_t)G * n, vc);
      load_vec_smem<T, K>(st + 3 * (size_t)G * n, vd);
      release_stage(&empty[s]);
    } else {
      const long base = sys * n + (long)t * K;
#pragma unroll
      for (int i = 0; i < K; ++i) {
        const bool in = sys < p.m;
        va[i] = in ? ga[base + i] : T(0);
        vb[i] = in ? gb[base + i] : T(1);
        vc[i] = in ? gc[base + i] : T(0);
        vd[i] = in ? gd[base + i] : T(0);
      }
    }
#pragma unroll
    for (int i = 0; i < K; ++i) r[i] = Row<T>{va[i], vb[i], vc[i], vd[i]};
    T xr[K];
    hybrid_solve<T, K, WARP, LSTRIDE>(r, xr, t, tps, p.stride, sc, exports, ct);
    if (sys < p.m) {
      T* dst = gx + sys * n + (long)t * K;
      if (S > 0) store_vec<T, K>(dst, xr);
      else {
#pragma unroll
        for (int i = 0; i < K; ++i) dst[i] = xr[i];
      }
    }
  }
  (void)LOGK;
}

// Warp shapes (a system's group fits in one warp) without a producer warp:
// every warp streams its own systems through a private two-buffer ring.
// While a warp solves warp tile k (32 / tps systems, loaded from its buffer
// into registers), the bulk copies of its next tile fill the other buffer.
// No CTA barrier and no producer warp: all resident warps solve, so more of
// them fit an SM at the same register budget.  Needs the bulk-copy
// alignment (16-byte pointers, n * sizeof(T) a multiple of 16).
template <class T, int K, int LSTRIDE, int MINB>
__global__ void __launch_bounds__(kWarpKernelThreads, MINB) hybrid_warp_kernel(HybridParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = p.n, tps = p.tps;
  const int gw = 32 / tps;  // systems per warp tile
  const size_t buf_elems = (size_t)4 * gw * n;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + 2 * warp;
  T* buf = reinterpret_cast<T*>(smem + HybridSmem<T>::barrier_bytes()) + (size_t)2 * warp * buf_elems;
  const T* ga = static_cast<const T*>(p.a);
  const T* gb = static_cast<const T*>(p.b);
  const T* gc = static_cast<const T*>(p.c);
  const T* gd = static_cast<const T*>(p.d);
  T* gx = static_cast<T*>(p.x);
  const long tiles = ((long)p.m + gw - 1) / gw;
  const long first = (long)blockIdx.x * (blockDim.x >> 5) + warp;
  const long step = (long)gridDim.x * (blockDim.x >> 5);
  if (lane == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  __syncwarp();
  const auto issue = [&](long tile, int s) {  // lane 0
    const long sys0 = tile * gw;
    const long ns = (p.m - sys0) < gw ? (p.m - sys0) : gw;
    const uint32_t bytes = (uint32_t)(ns * n * sizeof(T));
    T* st = buf + s * buf_elems;
    mbar_arrive_expect_tx(&bars[s], 4 * bytes);
    bulk_g2s(st + 0 * (size_t)gw * n, ga + sys0 * n, bytes, &bars[s]);
    bulk_g2s(st + 1 * (size_t)gw * n, gb + sys0 * n, bytes, &bars[s]);
    bulk_g2s(st + 2 * (size_t)gw * n, gc + sys0 * n, bytes, &bars[s]);
    bulk_g2s(st + 3 * (size_t)gw * n, gd + sys0 * n, bytes, &bars[s]);
  };
  if (lane == 0 && first < tiles) issue(first, 0);
  const int g = lane / tps, t = lane - g * tps;
  int k = 0;
  for (long tile = first; tile < tiles; tile += step, ++k) {
    const int s = k & 1;
    // the other buffer was read into registers one tile ago (and the warp
    // synchronised since): refill it with the next tile
    if (lane == 0 && tile + step < tiles) {
      fence_proxy_async_smem();
      issue(tile + step, s ^ 1);
    }
    if (!mbar_wait(&bars[s], (k >> 1) & 1, p.status)) break;
    const T* st = buf + s * buf_elems + (size_t)g * n + (size_t)t * K;
    T va[K], vb[K], vc[K], vd[K];
    load_vec_smem<T, K>(st + 0 * (size_t)gw * n, va);
    load_vec_smem<T, K>(st + 1 * (size_t)gw * n, vb);
    load_vec_smem<T, K>(st + 2 * (size_t)gw * n, vc);
    load_vec_smem<T, K>(st + 3 * (size_t)gw * n, vd);
    __syncwarp();
    Row<T> r[K];
#pragma unroll
    for (int i = 0; i < K; ++i) r[i] = Row<T>{va[i], vb[i], vc[i], vd[i]};
    T xr[K];
    hybrid_solve<T, K, true, LSTRIDE>(r, xr, t, tps, p.stride, GroupScratch<T>{}, nullptr, 32);
    const long sys = tile * gw + g;
    if (sys < p.m) store_vec<T, K>(gx + sys * n + (long)t * K, xr);
  }
}

// Block shapes (a system's group spans several warps) without a producer
// warp: the CTA is one or more groups (ct = max(tps, 128) threads), every
// thread solves, and thread 0 streams the CTA's tiles through a two-buffer
// ring: tiles k and k+1 are in flight while tile k is read into registers;
// after a CTA barrier (everyone has read buffer s) tile k+2 is issued into
// it, then the solve runs.  Same arithmetic as hybrid_kernel.
template <class T, int K, int LSTRIDE, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) hybrid_block_stream_kernel(HybridParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  const int n = p.n, G = p.G, tps = p.tps, ct = p.ct;
  T* stages = reinterpret_cast<T*>(smem + HybridSmem<T>::barrier_bytes());
  const size_t stage_elems = HybridSmem<T>::stage_elems(G, n);
  const int tid = threadIdx.x;
  const T* ga = static_cast<const T*>(p.a);
  const T* gb = static_cast<const T*>(p.b);
  const T* gc = static_cast<const T*>(p.c);
  const T* gd = static_cast<const T*>(p.d);
  T* gx = static_cast<T*>(p.x);
  const auto issue = [&](int tile, int s) {  // thread 0
    const long sys0 = (long)tile * G;
    const long nsys = (p.m - sys0) < G ? (p.m - sys0) : G;
    const uint32_t bytes = (uint32_t)(nsys * n * sizeof(T));
    T* st = stages + s * stage_elems;
    mbar_arrive_expect_tx(&bars[s], 4 * bytes);
    bulk_g2s(st + 0 * (size_t)G * n, ga + sys0 * n, bytes, &bars[s]);
    bulk_g2s(st + 1 * (size_t)G * n, gb + sys0 * n, bytes, &bars[s]);
    bulk_g2s(st + 2 * (size_t)G * n, gc + sys0 * n, bytes, &bars[s]);
    bulk_g2s(st + 3 * (size_t)G * n, gd + sys0 * n, bytes, &bars[s]);
  };
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
    if ((int)blockIdx.x < p.ntiles) issue(blockIdx.x, 0);
    if ((int)(blockIdx.x + gridDim.x) < p.ntiles) issue(blockIdx.x + gridDim.x, 1);
  }
  __syncthreads();

  const int g = tid / tps;
  const int t = tid - g * tps;
  T* base = stages + 2 * stage_elems;
  const size_t rows = p.scratch_rows;
  T* mine = base + (size_t)g * 5 * rows;
  const GroupScratch<T> sc{mine, mine + rows, mine + 2 * rows, mine + 3 * rows, mine + 4 * rows};
  Row<T>* exports = reinterpret_cast<Row<T>*>(base + (size_t)G * 5 * rows);
  int k = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
    const int s = k & 1;
    const bool ok = consumer_sync_and(ct, mbar_wait(&bars[s], (k >> 1) & 1, p.status));
    if (!ok) break;
    const T* st = stages + s * stage_elems + (size_t)g * n + (size_t)t * K;
    T va[K], vb[K], vc[K], vd[K];
    load_vec_smem<T, K>(st + 0 * (size_t)G * n, va);
    load_vec_smem<T, K>(st + 1 * (size_t)G * n, vb);
    load_vec_smem<T, K>(st + 2 * (size_t)G * n, vc);
    load_vec_smem<T, K>(st + 3 * (size_t)G * n, vd);
    consumer_sync(ct);  // buffer s read by every thread
    if (tid == 0 && tile + 2 * (int)gridDim.x < p.ntiles) {
      fence_proxy_async_smem();
      issue(tile + 2 * gridDim.x, s);
    }
    Row<T> r[K];
#pragma unroll
    for (int i = 0; i < K; ++i) r[i] = Row<T>{va[i], vb[i], vc[i], vd[i]};
    T xr[K];
    hybrid_solve<T, K, false, LSTRIDE>(r, xr, t, tps, p.stride, sc, exports, ct);
    const long sys = (long)tile * G + g;
    if (sys < p.m) store_vec<T, K>(gx + sys * n + (long)t * K, xr);
  }
}

}  // namespace tridi

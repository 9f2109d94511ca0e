// Partition solver: the GB300 engine for systems of any size (not only powers
// of two), used by the generic solve, the large-system and ragged paths and
// the refinement loop.  It has no counterpart kernel in the reference; its
// oracle is the same gold Thomas solver (tridiagonal_gold.h:26-44).
//
// A system's rows are cut into contiguous chunks, one per lane (thread).  The
// last row of chunk j is its separator s_j; the other rows are interior.
//   1. Chunk elimination (sequential, in registers): a downward Thomas-like
//      sweep over the interior rows gives, per row i,
//          x_i + c'_i x_{i+1} + a'_i s_{j-1} = d'_i
//      (one reciprocal and six flops per row).  A division-free upward pass
//      expresses the first interior row as x = D - C s_j - A s_{j-1}; the
//      last interior row is already in that form.
//   2. Separator system: substituting the neighbouring interior rows into the
//      separator's equation couples s_j to s_{j-1} and s_{j+1} only: a
//      tridiagonal system with one row per lane, solved by PCR over the warp's
//      lanes (shuffles; lanes past the system are identity rows).
//   3. Back substitution: x_{k-1} = s_j, x_i = d'_i - c'_i x_{i+1} - a'_i s_{j-1}.
// a[0] and c[n-1] are ignored (treated as zero), as the gold solver does.
//
// Lanes own an odd number of rows (kk), so lane l reading row l*kk + i of a
// dense shared-memory copy of the system hits 32 distinct banks.
#pragma once
#include "tridi_device.cuh"

namespace tridi {

template <class T, int K>
struct Chunk {
  T cp[K], ap[K], dp[K];  // normalised downward elimination of the interior rows
  Row<T> sep;             // separator row (the chunk's last row)
  T fD, fC, fA;           // first interior row:  x = fD - fC s_j - fA s_{j-1}
  T lD, lC, lA;           // last interior row (row k-2), same form
};

// Eliminates the lane's k rows (0 <= k <= K), row i of the chunk being
// (pa[i*rs], pb[i*rs], pc[i*rs], pd[i*rs]).  first/last: the chunk holds the
// system's first/last row.
// PREFETCH (for global-memory rows): all k rows are loaded into registers
// before the dependent elimination chain starts, so their loads overlap.
template <class T, int K, bool PREFETCH = false>
__device__ __forceinline__ void chunk_eliminate(Chunk<T, K>& ch, int k, bool first, bool last, const T* pa,
                                                const T* pb, const T* pc, const T* pd, long rs = 1) {
  T qa[PREFETCH ? K : 1], qb[PREFETCH ? K : 1], qc[PREFETCH ? K : 1], qd[PREFETCH ? K : 1];
  if constexpr (PREFETCH) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
      if (i < k - 1) {
        qa[i] = pa[i * rs]; qb[i] = pb[i * rs]; qc[i] = pc[i * rs]; qd[i] = pd[i * rs];
      }
    }
  }
  T cprev = T(0), aprev = T(0), dprev = T(0);
#pragma unroll
  for (int i = 0; i < K; ++i) {
    if (i < k - 1) {
      const Row<T> r = PREFETCH ? Row<T>{qa[PREFETCH ? i : 0], qb[PREFETCH ? i : 0], qc[PREFETCH ? i : 0],
                                         qd[PREFETCH ? i : 0]}
                                : Row<T>{pa[i * rs], pb[i * rs], pc[i * rs], pd[i * rs]};
      const T a = (i == 0 && first) ? T(0) : r.a;
      const T inv = tdiv(T(1), r.b - a * cprev);
      ch.cp[i] = r.c * inv;
      ch.ap[i] = (i == 0 ? a : -a * aprev) * inv;
      ch.dp[i] = (r.d - a * dprev) * inv;
      cprev = ch.cp[i];
      aprev = ch.ap[i];
      dprev = ch.dp[i];
    }
  }
  // Upward, division free: coefficients of the first interior row.  Seeded
  // with the separator itself (x_{k-1} = s_j: D = 0, C = -1, A = 0), so the
  // step at row k-2 yields exactly (d', c', a') of that row, and a chunk with
  // no interior row keeps (0, -1, 0): the row after the left separator is s_j.
  T D = T(0), C = T(-1), A = T(0);
#pragma unroll
  for (int i = K - 1; i >= 0; --i) {
    if (i <= k - 2) {
      D = ch.dp[i] - ch.cp[i] * D;
      C = -ch.cp[i] * C;
      A = ch.ap[i] - ch.cp[i] * A;
    }
  }
  ch.fD = D; ch.fC = C; ch.fA = A;
  if (k >= 2) {
    ch.lD = dprev; ch.lC = cprev; ch.lA = aprev;
  } else {  // no interior row: the row before the separator is s_{j-1}
    ch.lD = T(0); ch.lC = T(0); ch.lA = T(-1);
  }
  if (k >= 1) {
    const long o = (long)(k - 1) * rs;
    ch.sep = Row<T>{pa[o], pb[o], pc[o], pd[o]};
    if (k == 1 && first) ch.sep.a = T(0);
    if (last) ch.sep.c = T(0);
  } else {  // lane past the end of the system: identity separator
    ch.sep = Row<T>{T(0), T(1), T(0), T(0)};
  }
}

// Summary of a chunk eliminated in shared memory: what the separator system
// and the back substitution need besides the rows themselves.
template <class T>
struct ChunkSummary {
  Row<T> sep;
  T fD, fC, fA;
  T lD, lC, lA;
};

// The right-hand side of row i as staged (rhs(i, a, b, c, d) = d).  A
// right-hand side functor is told the chunk's first row (start) and then
// called for the chunk's rows in order.
struct RhsStaged {
  static constexpr bool kPairs = false;  // true: pair(i, row i, row i + 1) gives two rows' right-hand sides
  __device__ __forceinline__ void start(int) const {}
  template <class T>
  __device__ __forceinline__ T operator()(int, T, T, T, T d) const {
    return d;
  }
};

// chunk_eliminate on rows held in shared memory (no size bound, K-free):
// interior rows i < k-1 get (a, c, d) overwritten by (ap, cp, dp), so the
// back substitution reads them again instead of holding 3k registers.
// Row i's right-hand side is rhs(i, a_i, b_i, c_i, d_i) of its staged values
// (a correction solve forms its residual there, as the row is eliminated).
template <class T, class Rhs = RhsStaged>
__device__ __forceinline__ void chunk_eliminate_smem(ChunkSummary<T>& cs, int k, bool first, bool last,
                                                     T* __restrict__ sa, const T* __restrict__ sb,
                                                     T* __restrict__ sc, T* __restrict__ sd,
                                                     const Rhs& rhs = Rhs()) {
  T cprev = T(0), aprev = T(0), dprev = T(0);
  const auto step = [&](int i, T a0, T b0, T c0, T r) {
    const T a = (i == 0 && first) ? T(0) : a0;
    const T inv = tdiv(T(1), b0 - a * cprev);
    const T cn = c0 * inv;
    const T an = (i == 0 ? a : -a * aprev) * inv;
    const T dn = (r - a * dprev) * inv;
    sa[i] = an; sc[i] = cn; sd[i] = dn;
    cprev = cn; aprev = an; dprev = dn;
  };
  if constexpr (Rhs::kPairs) {
    // the right-hand sides of rows i and i + 1 formed together (they do not
    // depend on the elimination), the two rows then eliminated in order
    int i = 0;
#pragma unroll 2
    for (; i + 1 < k - 1; i += 2) {
      const T a0 = sa[i], b0 = sb[i], c0 = sc[i], d0 = sd[i];
      const T a1 = sa[i + 1], b1 = sb[i + 1], c1 = sc[i + 1], d1 = sd[i + 1];
      const auto r = rhs.pair(i, a0, b0, c0, d0, a1, b1, c1, d1);
      step(i, a0, b0, c0, r.x);
      step(i + 1, a1, b1, c1, r.y);
    }
    if (i < k - 1) {
      const T a0 = sa[i], b0 = sb[i], c0 = sc[i];
      step(i, a0, b0, c0, rhs(i, a0, b0, c0, sd[i]));
    }
  } else {
#pragma unroll 4
    for (int i = 0; i < k - 1; ++i) {
      const T a0 = sa[i], b0 = sb[i], c0 = sc[i];
      step(i, a0, b0, c0, rhs(i, a0, b0, c0, sd[i]));
    }
  }
  T D = T(0), C = T(-1), A = T(0);
#pragma unroll 4
  for (int i = k - 2; i >= 0; --i) {
    const T c = sc[i];
    D = sd[i] - c * D;
    C = -c * C;
    A = sa[i] - c * A;
  }
  cs.fD = D; cs.fC = C; cs.fA = A;
  if (k >= 2) {
    cs.lD = dprev; cs.lC = cprev; cs.lA = aprev;
  } else {
    cs.lD = T(0); cs.lC = T(0); cs.lA = T(-1);
  }
  if (k >= 1) {
    const T a0 = sa[k - 1], b0 = sb[k - 1], c0 = sc[k - 1];
    cs.sep = Row<T>{a0, b0, c0, rhs(k - 1, a0, b0, c0, sd[k - 1])};
    if (k == 1 && first) cs.sep.a = T(0);
    if (last) cs.sep.c = T(0);
  } else {
    cs.sep = Row<T>{T(0), T(1), T(0), T(0)};
  }
}

template <class T>
__device__ __forceinline__ Row<T> separator_row_s(const ChunkSummary<T>& cs, T nD, T nC, T nA) {
  const Row<T>& s = cs.sep;
  return Row<T>{-s.a * cs.lA, s.b - s.a * cs.lC - s.c * nA, -s.c * nC, s.d - s.a * cs.lD - s.c * nD};
}

// Back substitution of a chunk eliminated by chunk_eliminate_smem: emit(i, x_i)
// for every row i < k of the chunk, last row first.
// (emit writes to arrays other than sa, sc, sd.)
template <class T, class Emit>
__device__ __forceinline__ void chunk_back_smem(int k, T sj, T sl, const T* __restrict__ sa,
                                                const T* __restrict__ sc, const T* __restrict__ sd, Emit& emit) {
  if (k >= 1) emit(k - 1, sj);
  T xn = sj;
#pragma unroll 4
  for (int i = k - 2; i >= 0; --i) {
    xn = sd[i] - sc[i] * xn - sa[i] * sl;
    emit(i, xn);
  }
}

// Same, with x_i written over the chunk's d_i (row i's d is read once, by
// the step that produces x_i).
template <class T>
__device__ __forceinline__ void chunk_back_smem_over_d(int k, T sj, T sl, const T* __restrict__ sa,
                                                       const T* __restrict__ sc, T* __restrict__ sd) {
  if (k >= 1) sd[k - 1] = sj;
  T xn = sj;
#pragma unroll 4
  for (int i = k - 2; i >= 0; --i) {
    xn = sd[i] - sc[i] * xn - sa[i] * sl;
    sd[i] = xn;
  }
}

// The lane's row of the separator system, given the next chunk's first
// interior row (nD, nC, nA).
template <class T, int K>
__device__ __forceinline__ Row<T> separator_row(const Chunk<T, K>& ch, T nD, T nC, T nA) {
  const Row<T>& s = ch.sep;
  return Row<T>{-s.a * ch.lA, s.b - s.a * ch.lC - s.c * nA, -s.c * nC, s.d - s.a * ch.lD - s.c * nD};
}

// PCR over the 32 lanes of a warp (one row per lane, identity rows outside):
// returns the lane's unknown.
template <class T>
__device__ __forceinline__ T warp_pcr32(Row<T> r) {
  const int lane = threadIdx.x & 31;
  const Row<T> id{T(0), T(1), T(0), T(0)};
#pragma unroll
  for (int dl = 1; dl < 32; dl *= 2) {
    Row<T> L = shfl_up(r, dl, 32);
    Row<T> R = shfl_down(r, dl, 32);
    if (lane < dl) L = id;
    if (lane + dl > 31) R = id;
    r = reduce_row(r, L, R);
  }
  return tdiv(r.d, r.b);
}

// Back substitution of the lane's chunk: sj its separator, sl the left one.
template <class T, int K>
__device__ __forceinline__ void chunk_back(const Chunk<T, K>& ch, int k, T sj, T sl, T (&x)[K]) {
  T xn = sj;
#pragma unroll
  for (int i = K - 1; i >= 0; --i) {
    xn = (i <= k - 2) ? ch.dp[i] - ch.cp[i] * xn - ch.ap[i] * sl : sj;
    x[i] = xn;
  }
}

// Same, handing each unknown to emit(i, x_i) (i < k) as soon as it is known.
template <class T, int K, class Emit>
__device__ __forceinline__ void chunk_back_emit(const Chunk<T, K>& ch, int k, T sj, T sl, Emit& emit) {
  T xn = sj;
#pragma unroll
  for (int i = K - 1; i >= 0; --i) {
    xn = (i <= k - 2) ? ch.dp[i] - ch.cp[i] * xn - ch.ap[i] * sl : sj;
    if (i < k) emit(i, xn);
  }
}

// Whole system in one warp: lane l owns rows [l*kk, min(l*kk+kk, n)) of the
// arrays (sa, sb, sc, sd).  Returns the lane's row count.
template <class T, int K>
__device__ __forceinline__ int warp_partition_solve(int n, int kk, const T* sa, const T* sb, const T* sc,
                                                    const T* sd, T (&x)[K]) {
  const int lane = threadIdx.x & 31;
  const int r0 = lane * kk;
  int k = n - r0;
  k = k < 0 ? 0 : (k > kk ? kk : k);
  Chunk<T, K> ch;
  chunk_eliminate<T, K>(ch, k, lane == 0, r0 + k == n && k > 0, sa + r0, sb + r0, sc + r0, sd + r0);
  const T nD = __shfl_down_sync(kFull, ch.fD, 1);
  const T nC = __shfl_down_sync(kFull, ch.fC, 1);
  const T nA = __shfl_down_sync(kFull, ch.fA, 1);
  const T s = warp_pcr32<T>(separator_row<T, K>(ch, nD, nC, nA));
  T sl = __shfl_up_sync(kFull, s, 1);
  if (lane == 0) sl = T(0);
  chunk_back<T, K>(ch, k, s, sl, x);
  return k;
}

}  // namespace tridi

// Bank-conflict-free shared-memory cyclic reduction (crNBC, crNBC32,
// crpcrNBC) for sm_103a.
//
// The reference pads its shared arrays (crNBC.cu:8-17, one word per 16 for
// GT200's 16 banks; crNBC32banks.cu:8-17 meant one per 32 but is the
// identity) so that the stride-2^j accesses of CR collide less.  Padding
// only helps some levels.  Here every level is conflict-free for the 32
// banks of the GB300 by construction: each forward level writes the rows it
// eliminates into a new, dense array (level l+1 holds the odd rows of level
// l), so at every level thread j touches rows 2j, 2j+1 (one 8- or 16-byte
// pair load: conflict-free) and 2j+2 (the next lane's pair, by shuffle).
// Back substitution walks the levels in reverse with the same pattern and
// writes x pairwise; level 0 writes x straight to global memory, coalesced.
//
// One warp solves one system; a tile holds G systems (one per consumer
// warp) and arrives through the same cp.async.bulk + mbarrier ring as the
// register kernels.  The stage is the level-0 array, so it is released only
// after the warp's solve.  Arithmetic: reduce_row / solve2_* / back_row, the
// reference's formulas (crNBC.cu:68-73, :86-88, :107-110; the hybrid's PCR
// :268-307).
#pragma once
#include "tridi_device.cuh"

namespace tridi {

struct NbcParams {
  const void* a;
  const void* b;
  const void* c;
  const void* d;
  void* x;
  int n;
  int m;
  int G;        // systems (warps) per tile
  int ntiles;
  int rest;     // size of the PCR-solved intermediate system (2 = plain CR)
  int stages;   // 0 = level 0 read straight from global memory
  int vec;      // 1 if global x and level-0 arrays allow pair accesses
  unsigned* status;
};

template <class T>
struct NbcSmem {
  // per group: 4 coefficient regions of n (levels >= 1), an x region of n
  // (levels >= 1), and a 4*rest PCR ping-pong buffer.
  static __host__ __device__ size_t group_elems(int n, int rest) { return (size_t)5 * n + 4 * (size_t)rest; }
  static __host__ __device__ size_t bytes(int stages, int G, int n, int rest) {
    return 128 + (size_t)stages * 4 * G * n * sizeof(T) + (size_t)G * group_elems(n, rest) * sizeof(T);
  }
};

template <class T>
struct Pair {
  T lo, hi;
};

template <class T>
__device__ __forceinline__ Pair<T> load_pair(const T* p, int i, bool vec) {
  if (vec) {
    if constexpr (sizeof(T) == 4) {
      const float2 v = *reinterpret_cast<const float2*>(p + i);
      return {v.x, v.y};
    } else {
      const double2 v = *reinterpret_cast<const double2*>(p + i);
      return {v.x, v.y};
    }
  }
  return {p[i], p[i + 1]};
}
template <class T>
__device__ __forceinline__ void store_pair(T* p, int i, T lo, T hi, bool vec) {
  if (vec) {
    if constexpr (sizeof(T) == 4) *reinterpret_cast<float2*>(p + i) = make_float2(lo, hi);
    else *reinterpret_cast<double2*>(p + i) = make_double2(lo, hi);
  } else {
    p[i] = lo;
    p[i + 1] = hi;
  }
}

// The last CR levels of one system in registers: the level's nl <= 32 rows
// (ca..cd) one per lane, the rows (t + 1) % 2D == 0 reduced against the rows
// D away over shuffles until two remain, their 2x2 solve, then back
// substitution the same way; x of the level's rows lands in xo.  The same
// formulas in the same order as the shared-memory levels (the odd rows of
// one level are the rows (t + 1) % 2D == 0 of the next finer spacing).
template <class T>
__device__ __forceinline__ void register_tail(const T* ca, const T* cb, const T* cc, const T* cd, T* xo, int nl,
                                              int lane) {
  const int t = lane;
  Row<T> C = t < nl ? Row<T>{ca[t], cb[t], cc[t], cd[t]} : Row<T>{T(0), T(1), T(0), T(0)};
  for (int D = 1; 2 * D < nl; D *= 2) {
    const Row<T> L = shfl_up(C, D, 32);
    Row<T> R = shfl_down(C, D, 32);
    if (t == nl - 1) R = C;  // right neighbour clamped to the last row (cr_kernel.cu:52)
    if (t < nl && ((t + 1) & (2 * D - 1)) == 0) C = reduce_row(C, L, R);
  }
  T xC = T(0);
  const Row<T> pr = shfl_xor(C, nl / 2, 32);
  if (t == nl / 2 - 1) xC = solve2_upper(C, pr);
  if (t == nl - 1) xC = solve2_lower(pr, C);
  for (int D = nl / 4; D >= 1; D /= 2) {
    const T xl = __shfl_up_sync(kFull, xC, D);
    const T xr = __shfl_down_sync(kFull, xC, D);
    if (t < nl && ((t + 1) & (2 * D - 1)) == D) xC = back_row(C, xl, xr, t == D - 1);
  }
  if (t < nl) xo[t] = xC;
}

// One system, one warp.  (la, lb, lc, ld): level-0 arrays (shared stage or
// global); W: the warp's working area; xg: the system's x in global memory.
template <class T>
__device__ void nbc_solve(const T* la, const T* lb, const T* lc, const T* ld, T* W, T* xg, int n, int rest,
                          bool vec0, bool vecx) {
  const int lane = threadIdx.x & 31;
  T* A = W;
  T* B = W + n;
  T* C = W + 2 * n;
  T* D = W + 3 * n;
  T* X = W + 4 * n;
  T* P = W + 5 * n;  // PCR ping-pong, 4 * rest

  // ---- forward CR levels: level l (nl rows) -> level l+1 (nl/2 rows) ----
  // Plain CR (rest == 2) leaves the shared-memory levels at 32 rows: one row
  // per lane, the remaining levels in registers (register_tail).
  const int stop = rest == 2 ? 32 : rest;
  const T *sa = la, *sb = lb, *sc = lc, *sd = ld;
  bool svec = vec0;
  int nl = n;
  while (nl > stop) {
    const int half = nl / 2;
    const int off = n - nl;  // offset of level l+1 (n - 2 * (nl/2))
    // level l is read, level l+1 written: disjoint arrays, so the iterations'
    // loads may run ahead of the previous iterations' stores
    const T* __restrict__ ra = sa;
    const T* __restrict__ rb = sb;
    const T* __restrict__ rc = sc;
    const T* __restrict__ rd = sd;
    T* __restrict__ wa = A + off;
    T* __restrict__ wb = B + off;
    T* __restrict__ wc = C + off;
    T* __restrict__ wd = D + off;
#pragma unroll 2
    for (int j0 = 0; j0 < half; j0 += 32) {
      const int j = j0 + lane;
      const int jj = j < half ? j : half - 1;
      const Pair<T> pa = load_pair(ra, 2 * jj, svec), pb = load_pair(rb, 2 * jj, svec),
                    pc = load_pair(rc, 2 * jj, svec), pd = load_pair(rd, 2 * jj, svec);
      Row<T> R{__shfl_down_sync(kFull, pa.lo, 1), __shfl_down_sync(kFull, pb.lo, 1),
               __shfl_down_sync(kFull, pc.lo, 1), __shfl_down_sync(kFull, pd.lo, 1)};
      const Row<T> me{pa.hi, pb.hi, pc.hi, pd.hi};
      if (jj == half - 1) {
        R = me;  // right neighbour clamped to the last row (cr_kernel.cu:52)
      } else if (lane == 31) {
        const int k = 2 * jj + 2;
        R = Row<T>{ra[k], rb[k], rc[k], rd[k]};
      }
      const Row<T> o = reduce_row(me, Row<T>{pa.lo, pb.lo, pc.lo, pd.lo}, R);
      if (j < half) {
        wa[j] = o.a; wb[j] = o.b; wc[j] = o.c; wd[j] = o.d;
      }
    }
    __syncwarp();
    sa = A + off; sb = B + off; sc = C + off; sd = D + off;
    svec = true;
    nl = half;
  }

  T* xl = (nl == n) ? nullptr : X + (n - 2 * nl);  // x of the intermediate level
  if (rest == 2) {
    register_tail<T>(sa, sb, sc, sd, xl ? xl : xg, nl, lane);
  } else {
  // ---- the intermediate system (nl == rest rows): PCR, then 2x2 pairs ----
    const T *ca = sa, *cb = sb, *cc = sc, *cd = sd;
    T *pa = P, *pb = P + rest, *pc = P + 2 * rest, *pd = P + 3 * rest;
    T *qa = const_cast<T*>(sa), *qb = const_cast<T*>(sb), *qc = const_cast<T*>(sc), *qd = const_cast<T*>(sd);
    for (int dl = 1; 4 * dl <= nl; dl *= 2) {  // rest/2 > 1 only for the hybrid
      for (int j = lane; j < nl; j += 32) {
        const int jl = j - dl < 0 ? 0 : j - dl;
        const int jr = j + dl > nl - 1 ? nl - 1 : j + dl;
        const Row<T> o = reduce_row(Row<T>{ca[j], cb[j], cc[j], cd[j]}, Row<T>{ca[jl], cb[jl], cc[jl], cd[jl]},
                                    Row<T>{ca[jr], cb[jr], cc[jr], cd[jr]});
        pa[j] = o.a; pb[j] = o.b; pc[j] = o.c; pd[j] = o.d;
      }
      __syncwarp();
      ca = pa; cb = pb; cc = pc; cd = pd;
      T *ta = pa, *tb = pb, *tc = pc, *td = pd;
      pa = qa; pb = qb; pc = qc; pd = qd;
      qa = ta; qb = tb; qc = tc; qd = td;
    }
    const int h = nl / 2;
    for (int j = lane; j < h; j += 32) {
      const Row<T> r1{ca[j], cb[j], cc[j], cd[j]};
      const Row<T> r2{ca[j + h], cb[j + h], cc[j + h], cd[j + h]};
      const T x1 = solve2_upper(r1, r2), x2 = solve2_lower(r1, r2);
      if (xl) {
        xl[j] = x1;
        xl[j + h] = x2;
      } else {  // n == rest == 2: the whole system was a 2x2
        xg[j] = x1;
        xg[j + h] = x2;
      }
    }
  }
  __syncwarp();

  // ---- back substitution: level l+1 x -> level l x, down to level 0 ----
  while (nl < n) {
    const int nu = nl * 2;  // rows of level l
    const T *ra, *rb, *rc, *rd;
    bool rvec;
    if (nu == n) {
      ra = la; rb = lb; rc = lc; rd = ld; rvec = vec0;
    } else {
      const int o = n - 2 * nu;
      ra = A + o; rb = B + o; rc = C + o; rd = D + o; rvec = true;
    }
    // x of level l+1 (odd rows of level l) is read, x of level l written
    const T* __restrict__ xo_arr = X + (n - 2 * nl);
    T* __restrict__ xe_arr = (nu == n) ? xg : X + (n - 2 * nu);
    const bool xvec = (nu == n) ? vecx : true;
#pragma unroll 2
    for (int j0 = 0; j0 < nl; j0 += 32) {
      const int j = j0 + lane;
      const int jj = j < nl ? j : nl - 1;
      const T xo = xo_arr[jj];
      T xprev = __shfl_up_sync(kFull, xo, 1);
      if (lane == 0) xprev = jj > 0 ? xo_arr[jj - 1] : T(0);
      const Pair<T> pa = load_pair(ra, 2 * jj, rvec), pb = load_pair(rb, 2 * jj, rvec),
                    pc = load_pair(rc, 2 * jj, rvec), pd = load_pair(rd, 2 * jj, rvec);
      const T xe = back_row(Row<T>{pa.lo, pb.lo, pc.lo, pd.lo}, xprev, xo, jj == 0);
      if (j < nl) store_pair(xe_arr, 2 * j, xe, xo, xvec);
    }
    __syncwarp();
    nl = nu;
  }
}

template <class T, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) nbc_kernel(NbcParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + 8;
  const int S = p.stages, n = p.n, G = p.G;
  const int ct = 32 * G;
  T* stages = reinterpret_cast<T*>(smem + 128);
  const size_t stage_elems = (size_t)4 * G * n;
  T* work = stages + (size_t)S * stage_elems;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;

  if (tid == 0 && S > 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], G);
    }
    mbar_fence_init();
  }
  __syncthreads();

  const T* ga = static_cast<const T*>(p.a);
  const T* gb = static_cast<const T*>(p.b);
  const T* gc = static_cast<const T*>(p.c);
  const T* gd = static_cast<const T*>(p.d);
  T* gx = static_cast<T*>(p.x);

  if (tid >= ct) {  // producer warp
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

  T* W = work + (size_t)warp * NbcSmem<T>::group_elems(n, p.rest);
  int k = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++k) {
    const long sys = (long)tile * G + warp;
    const T *la, *lb, *lc, *ld;
    bool vec0;
    int s = 0;
    if (S > 0) {
      s = k % S;
      if (!mbar_wait(&full[s], (k / S) & 1, p.status)) break;
      const T* st = stages + s * stage_elems + (size_t)warp * n;
      la = st; lb = st + (size_t)G * n; lc = st + 2 * (size_t)G * n; ld = st + 3 * (size_t)G * n;
      vec0 = true;
    } else {
      const long sc = sys < p.m ? sys : p.m - 1;
      la = ga + sc * n; lb = gb + sc * n; lc = gc + sc * n; ld = gd + sc * n;
      vec0 = false;
    }
    if (sys < p.m) nbc_solve<T>(la, lb, lc, ld, W, gx + sys * n, n, p.rest, vec0, p.vec != 0);
    if (S > 0) {
      release_stage(&empty[s]);
    }
  }
}

}  // namespace tridi

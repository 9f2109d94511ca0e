// Device-side building blocks shared by every solver kernel: the row type,
// the reduction formulas of the reference solvers, warp shuffles of rows,
// and the sm_103a asynchronous-copy machinery (mbarrier + cp.async.bulk) with
// bounded waits.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "tridi.h"

namespace tridi {

// Division used by every solver kernel.  FP32: the numerator times the
// hardware's approximate reciprocal of the divisor (PTX rcp.approx.ftz.f32,
// at most 1 ulp from 1/b; the product at most 2 ulp from the IEEE quotient),
// no slow-path branch and no range fix-up (divisors here are O(1), far from
// the denormal range that .ftz flushes).  FP64: the IEEE quotient.  Each
// division of the reference's formulas becomes one tdiv, so results stay
// within a few ulp of the reference's arithmetic.
__device__ __forceinline__ float rcp_approx(float v) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ float tdiv(float a, float b) { return a * rcp_approx(b); }
__device__ __forceinline__ double tdiv(double a, double b) { return a / b; }

// One equation a*x[i-1] + b*x[i] + c*x[i+1] = d.
template <class T>
struct Row {
  T a, b, c, d;
};

// Cyclic-reduction / PCR elimination of equation `me` against its two
// neighbours L (at i - delta) and R (at i + delta).  This is the update of
// the reference's solvers, written term for term in the same order so that
// the rounding matches: cr_kernel.cu:53-58, pcr_kernel.cu:39-56,
// crpcr_kernel.cu:50-55 and :92-98, crNBC.cu:68-73, pcrGauss_kernel.cu:89-98.
template <class T>
__device__ __forceinline__ Row<T> reduce_row(const Row<T>& me, const Row<T>& L, const Row<T>& R) {
  T tmp1 = tdiv(me.a, L.b);
  T tmp2 = tdiv(me.c, R.b);
  Row<T> o;
  o.b = me.b - L.c * tmp1 - R.a * tmp2;
  o.d = me.d - L.d * tmp1 - R.d * tmp2;
  o.a = -L.a * tmp1;
  o.c = -R.c * tmp2;
  return o;
}

// A row divided by its diagonal: (a/b, c/b, d/b).  In PCR every row is the
// divisor of both its neighbours at a step, so its owner divides once and
// hands them these three values (three shuffles instead of four).
template <class T>
struct NRow {
  T a, c, d;
};
template <class T>
__device__ __forceinline__ NRow<T> normalize_row(const Row<T>& r) {
  const T ib = tdiv(T(1), r.b);
  return {r.a * ib, r.c * ib, r.d * ib};
}

// reduce_row with the neighbours given as normalised rows:
// me - (me.a) L - (me.c) R, the same elimination up to rounding order.
template <class T>
__device__ __forceinline__ Row<T> reduce_row_nrm(const Row<T>& me, const NRow<T>& L, const NRow<T>& R) {
  Row<T> o;
  o.b = me.b - me.a * L.c - me.c * R.a;
  o.d = me.d - me.a * L.d - me.c * R.d;
  o.a = -me.a * L.a;
  o.c = -me.c * R.c;
  return o;
}

// The 2x2 solve that closes CR / PCR (cr_kernel.cu:65-69, pcr_kernel.cu:67-71):
// unknown 1 is the upper equation (r1), unknown 2 the lower (r2).
template <class T>
__device__ __forceinline__ T solve2_upper(const Row<T>& r1, const Row<T>& r2) {
  T tmp3 = r2.b * r1.b - r1.c * r2.a;
  return tdiv(r2.b * r1.d - r1.c * r2.d, tmp3);
}
template <class T>
__device__ __forceinline__ T solve2_lower(const Row<T>& r1, const Row<T>& r2) {
  T tmp3 = r2.b * r1.b - r1.c * r2.a;
  return tdiv(r2.d * r1.b - r1.d * r2.a, tmp3);
}

// Back substitution of one unknown from its solved neighbours
// (cr_kernel.cu:81-84).  `first` is the system's first row, which has no
// left neighbour term.
template <class T>
__device__ __forceinline__ T back_row(const Row<T>& r, T xl, T xr, bool first) {
  return first ? tdiv(r.d - r.c * xr, r.b) : tdiv(r.d - r.a * xl - r.c * xr, r.b);
}

// ---- warp shuffles of rows -------------------------------------------------
constexpr unsigned kFull = 0xffffffffu;

template <class T>
__device__ __forceinline__ NRow<T> shfl_up(const NRow<T>& v, int delta, int width) {
  return {__shfl_up_sync(kFull, v.a, delta, width), __shfl_up_sync(kFull, v.c, delta, width),
          __shfl_up_sync(kFull, v.d, delta, width)};
}
template <class T>
__device__ __forceinline__ NRow<T> shfl_down(const NRow<T>& v, int delta, int width) {
  return {__shfl_down_sync(kFull, v.a, delta, width), __shfl_down_sync(kFull, v.c, delta, width),
          __shfl_down_sync(kFull, v.d, delta, width)};
}

template <class T>
__device__ __forceinline__ Row<T> shfl_up(const Row<T>& v, int delta, int width) {
  return {__shfl_up_sync(kFull, v.a, delta, width), __shfl_up_sync(kFull, v.b, delta, width),
          __shfl_up_sync(kFull, v.c, delta, width), __shfl_up_sync(kFull, v.d, delta, width)};
}
template <class T>
__device__ __forceinline__ Row<T> shfl_down(const Row<T>& v, int delta, int width) {
  return {__shfl_down_sync(kFull, v.a, delta, width), __shfl_down_sync(kFull, v.b, delta, width),
          __shfl_down_sync(kFull, v.c, delta, width), __shfl_down_sync(kFull, v.d, delta, width)};
}
template <class T>
__device__ __forceinline__ Row<T> shfl_xor(const Row<T>& v, int mask, int width) {
  return {__shfl_xor_sync(kFull, v.a, mask, width), __shfl_xor_sync(kFull, v.b, mask, width),
          __shfl_xor_sync(kFull, v.c, mask, width), __shfl_xor_sync(kFull, v.d, mask, width)};
}
template <class T>
__device__ __forceinline__ Row<T> shfl_idx(const Row<T>& v, int src, int width) {
  return {__shfl_sync(kFull, v.a, src, width), __shfl_sync(kFull, v.b, src, width),
          __shfl_sync(kFull, v.c, src, width), __shfl_sync(kFull, v.d, src, width)};
}

// ---- named barrier among the consumer warps (barrier 0 is __syncthreads) ---
__device__ __forceinline__ void consumer_sync(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}
// Barrier with an AND reduction of `pred` over the consumer threads.
__device__ __forceinline__ bool consumer_sync_and(int nthreads, bool pred) {
  uint32_t out;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(out)
      : "r"((uint32_t)pred), "r"(nthreads)
      : "memory");
  return out != 0;
}

// ---- mbarrier + bulk async copy (sm_90+ PTX, used here for sm_103a) --------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's prior generic-proxy shared-memory accesses (ordinary
// ld.shared of a stage) before later async-proxy accesses (the next
// cp.async.bulk into the same stage).  Every consumer issues it before
// releasing a stage: without it a bulk copy of the next tile may overwrite
// rows that have not been read yet.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Release of a stage by one warp: fence, warp barrier, one arrive.
__device__ __forceinline__ void release_stage(uint64_t* bar) {
  fence_proxy_async_smem();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(bar)))
                 : "memory");
  }
}

// Same, the warp's arrive counting `count` arrivals.
__device__ __forceinline__ void release_stage_n(uint64_t* bar, uint32_t count) {
  fence_proxy_async_smem();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(bar))),
                 "r"(count)
                 : "memory");
  }
}

// Barrier with an AND reduction of `pred` over `nthreads` threads on named
// barrier `id`.
__device__ __forceinline__ bool named_sync_and(int id, int nthreads, bool pred) {
  uint32_t out;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(out)
      : "r"((uint32_t)pred), "r"(id), "r"(nthreads)
      : "memory");
  return out != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
                   smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Upper bound on any wait in these kernels, in SM clock cycles (~1 s at the
// GB300's 2 GHz maximum clock).  A wait that runs out records
// TRIDI_DEVERR_WAIT_TIMEOUT in the status word and returns false; the caller
// then stops issuing work and leaves the kernel.
constexpr long long kWaitLimitCycles = 2000000000LL;

__device__ __forceinline__ void record_error(unsigned* status, unsigned bit) {
  if (status) atomicOr(status, bit);
}

// Waits for the phase of `bar` with parity `parity` for at most
// `limit_cycles` SM cycles; on running out records TRIDI_DEVERR_WAIT_TIMEOUT
// and returns false.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, unsigned* status,
                                              long long limit_cycles) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit_cycles) {
      record_error(status, TRIDI_DEVERR_WAIT_TIMEOUT);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned* status) {
  return mbar_wait_for(bar, parity, status, kWaitLimitCycles);
}

// Bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from
// global to this CTA's shared memory; completion is signalled on `bar` as
// transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Tiled 2-D tensor copy (box at element coordinates x, y of `map`) from
// global to this CTA's shared memory, completion signalled on `bar`.  x times
// the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// ---- vector moves of K consecutive elements --------------------------------
// Loads/stores K consecutive T from/to `p` (16-byte aligned when K*sizeof(T)
// is a multiple of 16, which the callers guarantee) in 16-byte pieces.
template <class T, int K>
__device__ __forceinline__ void load_vec(const T* p, T (&v)[K]) {
  if constexpr ((K * sizeof(T)) % 16 == 0) {
    constexpr int PER = 16 / sizeof(T);
#pragma unroll
    for (int q = 0; q < K / PER; ++q) {
      if constexpr (sizeof(T) == 4) {
        float4 f = reinterpret_cast<const float4*>(p)[q];
        v[q * 4 + 0] = f.x; v[q * 4 + 1] = f.y; v[q * 4 + 2] = f.z; v[q * 4 + 3] = f.w;
      } else {
        double2 f = reinterpret_cast<const double2*>(p)[q];
        v[q * 2 + 0] = f.x; v[q * 2 + 1] = f.y;
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < K; ++q) v[q] = p[q];
  }
}

// load_vec from shared memory for threads whose K-element slices are
// consecutive (thread t at p = base + t*K): a 16-byte load of 8 threads is one
// shared-memory phase, and with slices 32 or 64 bytes apart their first
// chunks fall on the same banks (2- or 4-way conflicts).  Each thread
// starts at a different chunk of its slice, (q + t*Q/8) mod Q for Q chunks,
// so the 8 threads of a phase cover 8 distinct 16-byte bank groups.
template <class T, int K>
__device__ __forceinline__ void load_vec_smem(const T* p, T (&v)[K]) {
  constexpr int Q = (int)(K * sizeof(T) / 16);
  if constexpr (sizeof(T) == 4 && (K * sizeof(T)) % 16 == 0 && (Q == 2 || Q == 4)) {
    const int r = (int)((threadIdx.x * Q / 8) % Q);
    float4 f[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = reinterpret_cast<const float4*>(p)[(q + r) % Q];
    // chunk j is f[(j - r) mod Q]
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      float4 g = f[0];
#pragma unroll
      for (int q = 1; q < Q; ++q)
        if ((j - r + Q) % Q == q) g = f[q];
      v[4 * j + 0] = g.x; v[4 * j + 1] = g.y; v[4 * j + 2] = g.z; v[4 * j + 3] = g.w;
    }
  } else {
    load_vec<T, K>(p, v);
  }
}

template <class T, int K>
__device__ __forceinline__ void store_vec(T* p, const T (&v)[K]) {
  if constexpr ((K * sizeof(T)) % 16 == 0) {
    constexpr int PER = 16 / sizeof(T);
#pragma unroll
    for (int q = 0; q < K / PER; ++q) {
      if constexpr (sizeof(T) == 4) {
        reinterpret_cast<float4*>(p)[q] = make_float4(v[q * 4], v[q * 4 + 1], v[q * 4 + 2], v[q * 4 + 3]);
      } else {
        reinterpret_cast<double2*>(p)[q] = make_double2(v[q * 2], v[q * 2 + 1]);
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < K; ++q) p[q] = v[q];
  }
}

}  // namespace tridi

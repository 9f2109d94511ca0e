// Self-check of the bounded device waits: the path a wait takes when it runs
// out (status bit, early return), exercised on purpose without faulting or
// hanging the GPU.  One CTA waits on an mbarrier with an arrival count of 1;
// with `arrive` set, thread 0 arrives first and every wait completes; without
// it nothing ever arrives (and no bulk copy is issued into the barrier), so
// every thread's wait runs out after `limit_cycles` SM cycles, records
// TRIDI_DEVERR_WAIT_TIMEOUT in the device status word and returns.  The
// kernels' pipeline waits share this wait (mbar_wait, tridi_device.cuh) with
// the fixed limit of about one second.
#include "runtime.h"
#include "tridi_device.cuh"

namespace tridi {

__global__ void wait_selfcheck_kernel(long long limit_cycles, int arrive, unsigned* status, int* timed_out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0) mbar_arrive(&bar);
  const bool ok = mbar_wait_for(&bar, 0, status, limit_cycles);
  timed_out[threadIdx.x] = ok ? 0 : 1;
}

}  // namespace tridi

extern "C" tridi_status tridi_selfcheck_wait(long long limit_cycles, int arrive, int* timed_out, int num_threads,
                                             tridi_stream_t stream) {
  if (!timed_out || num_threads < 1 || num_threads > 1024 || limit_cycles < 1 ||
      limit_cycles > tridi::kWaitLimitCycles)
    return TRIDI_ERROR_INVALID_VALUE;
  const tridi::DeviceInfo* dev = tridi::current_device();
  if (!dev) return TRIDI_ERROR_CUDA;
  tridi::wait_selfcheck_kernel<<<1, num_threads, 0, tridi::as_stream(stream)>>>(limit_cycles, arrive ? 1 : 0,
                                                                                 dev->status, timed_out);
  return tridi::cuda_status(cudaGetLastError());
}

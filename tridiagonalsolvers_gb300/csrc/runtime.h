// Host-side runtime shared by every entry point: per-device facts (SM count,
// shared-memory limit), the per-device status word that bounded device waits
// report into, CUDA error capture, and the stream type conversion.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "tridi.h"

namespace tridi {

struct DeviceInfo {
  int device = -1;
  int sm_count = 0;
  int max_smem_optin = 0;   // bytes of dynamic shared memory a CTA may opt into
  unsigned* status = nullptr;  // device status word (TRIDI_DEVERR_* bits)
};

// Facts about the current device; allocates its status word on first use.
// Returns nullptr and sets the thread's CUDA error if the device cannot be
// queried.
const DeviceInfo* current_device();

// Records a CUDA error for tridi_last_cuda_error() and returns TRIDI_ERROR_CUDA
// (or TRIDI_SUCCESS for cudaSuccess).
tridi_status cuda_status(cudaError_t e);

inline cudaStream_t as_stream(tridi_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch-shape tunables (tridi_set_tunable); 0 means "choose automatically".
int tunable(int key);

// Set, on the calling thread, while a host-pointer launcher runs its kernels
// on host memory that the device maps (pinned, mapped arrays): the launches
// then read their inputs with plain loads, never with bulk or tensor copies.
extern thread_local bool g_host_mapped_io;

// Table written by the autotuner (tridi_autotune): per table (TRIDI_AUTOTUNE_*)
// and key (log2 of the system size, or of the size bucket), the chosen value;
// 0 where nothing was tuned.
int tuned(int table, int log2key);
// Ragged plans: the largest padded row count a warp or team item may hold
// (larger systems always take a whole CTA, whatever the threads table says).
long ragged_team_max_rows();
// PCR-then-Thomas in registers (pcr_thomas2.cu): whether it takes an FP32
// call, and the launch.
bool pcr_thomas2_applies(const void* a, const void* b, const void* c, const void* d, int n, long m, int g);
tridi_status pcr_thomas2_solve(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                               int m, int g, cudaStream_t stream);
// cr and crpcr at every switch level for 512 and 1024 unknowns, in registers
// (crpcr2.cu); stride = n / rest.
bool crpcr_regs_applies(const void* a, const void* b, const void* c, const void* d, const void* x, int n, long m,
                        int stride);
tridi_status crpcr_regs_solve(const float* a, const float* b, const float* c, const float* d, float* x, int n,
                              int m, int stride, cudaStream_t stream);

inline int ilog2(long v) {
  int k = 0;
  while (v > 1) {
    v >>= 1;
    ++k;
  }
  return k;
}

// Pipeline depth for a tiled kernel: the tunable if set, else `fallback`,
// reduced until the shared memory fits the device.
int pick_stages(size_t fixed_bytes, size_t stage_bytes, int fallback, const DeviceInfo& dev);

// A 2-D FP32 tensor map for cp.async.bulk.tensor: `outer` rows of `inner`
// elements, consecutive rows `row_bytes` apart, copied in boxes of
// box_inner x box_outer elements; swizzle128 selects the 128-byte swizzle
// (16-byte chunk c of box row r lands at chunk c ^ (r mod 8); the shared
// destination must then be 1024-byte aligned).  Out-of-range box elements
// read as zero.  False if the driver's encoder is unavailable or refuses the
// arguments.
bool make_tensor_map_2d(CUtensorMap* map, const float* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                        uint32_t box_inner, uint32_t box_outer, bool swizzle128);

// Largest system the uniform partition solver (tridi_solve_*) takes: 512
// threads of 17 rows (FP32) or 9 rows (FP64) each.
template <class T>
constexpr long partition_max_rows() {
  return sizeof(T) == 4 ? 512L * 17 : 512L * 9;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
inline bool is_pow2(long v) { return v > 0 && (v & (v - 1)) == 0; }

}  // namespace tridi

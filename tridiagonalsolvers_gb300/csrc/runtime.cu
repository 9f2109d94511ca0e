#include <cudaTypedefs.h>

#include <mutex>

#include "runtime.h"

namespace tridi {

namespace {
constexpr int kMaxDevices = 64;
DeviceInfo g_dev[kMaxDevices];
std::mutex g_mu;
thread_local int t_last_cuda_error = 0;
constexpr int kTunables = 13;
int g_tunable[kTunables] = {};
}  // namespace

thread_local bool g_host_mapped_io = false;

int tunable(int key) { return key >= 0 && key < kTunables ? g_tunable[key] : 0; }

namespace {
constexpr int kTuneTables = 5, kTuneKeys = 32;
int g_tuned[kTuneTables][kTuneKeys] = {};
}  // namespace

int tuned(int table, int log2key) {
  if (table < 0 || table >= kTuneTables || log2key < 0 || log2key >= kTuneKeys) return 0;
  return g_tuned[table][log2key];
}

int pick_stages(size_t fixed_bytes, size_t stage_bytes, int fallback, const DeviceInfo& dev) {
  int S = tunable(TRIDI_TUNE_STAGES);
  if (S <= 0) S = fallback;
  if (S > 8) S = 8;
  while (S > 1 && fixed_bytes + S * stage_bytes > (size_t)dev.max_smem_optin) --S;
  if (fixed_bytes + S * stage_bytes > (size_t)dev.max_smem_optin) S = 0;
  return S;
}

tridi_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return TRIDI_SUCCESS;
  t_last_cuda_error = static_cast<int>(e);
  return TRIDI_ERROR_CUDA;
}

const DeviceInfo* current_device() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cuda_status(e == cudaSuccess ? cudaErrorInvalidDevice : e);
    return nullptr;
  }
  DeviceInfo& d = g_dev[dev];
  if (d.status) return &d;
  std::lock_guard<std::mutex> lock(g_mu);
  if (d.status) return &d;
  int sms = 0, smem = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) {
    cuda_status(e);
    return nullptr;
  }
  unsigned* st = nullptr;
  if ((e = cudaMalloc(&st, 64)) != cudaSuccess || (e = cudaMemset(st, 0, 64)) != cudaSuccess) {
    cuda_status(e);
    return nullptr;
  }
  d.device = dev;
  d.sm_count = sms;
  d.max_smem_optin = smem;
  d.status = st;
  return &d;
}

namespace {
// The driver's tensor-map encoder, looked up through the runtime once (the
// library does not link the driver library itself, so it loads on machines
// without one).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}
}  // namespace

bool make_tensor_map_2d(CUtensorMap* map, const float* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                        uint32_t box_inner, uint32_t box_outer, bool swizzle128) {
  const auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
  const cuuint32_t box[2] = {box_inner, box_outer};
  const cuuint32_t elem[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tridi

using namespace tridi;

extern "C" {

const char* tridi_version(void) { return "tridi-gb300 0.1 (sm_103a)"; }

const char* tridi_status_string(tridi_status s) {
  switch (s) {
    case TRIDI_SUCCESS: return "success";
    case TRIDI_ERROR_INVALID_VALUE: return "invalid value";
    case TRIDI_ERROR_UNSUPPORTED_SIZE: return "unsupported system size";
    case TRIDI_ERROR_MISALIGNED: return "pointer not 16-byte aligned";
    case TRIDI_ERROR_CUDA: return "CUDA error";
    case TRIDI_ERROR_DEVICE_TIMEOUT: return "bounded device wait timed out";
    case TRIDI_ERROR_NOT_CONVERGED: return "iterative refinement did not converge";
    case TRIDI_ERROR_OUT_OF_MEMORY: return "out of memory";
    case TRIDI_ERROR_WORKSPACE_TOO_SMALL: return "workspace too small";
    case TRIDI_ERROR_BUSY: return "queue full";
  }
  return "unknown status";
}

int tridi_last_cuda_error(void) { return t_last_cuda_error; }

tridi_status tridi_set_tunable(int key, int value) {
  if (key < 0 || key >= kTunables || value < 0) return TRIDI_ERROR_INVALID_VALUE;
  g_tunable[key] = value;
  return TRIDI_SUCCESS;
}

int tridi_get_tunable(int key) { return tunable(key); }

int tridi_tuned(int table, long key) {
  if (key < 1) return 0;
  return tridi::tuned(table, tridi::ilog2(key));
}

tridi_status tridi_set_tuned(int table, long key, int value) {
  using namespace tridi;
  if (table < 0 || table >= kTuneTables || key < 1 || ilog2(key) >= kTuneKeys || value < 0)
    return TRIDI_ERROR_INVALID_VALUE;
  g_tuned[table][ilog2(key)] = value;
  return TRIDI_SUCCESS;
}

tridi_status tridi_autotune_reset(void) {
  for (auto& t : tridi::g_tuned)
    for (int& v : t) v = 0;
  return TRIDI_SUCCESS;
}

tridi_status tridi_init(void) { return current_device() ? TRIDI_SUCCESS : TRIDI_ERROR_CUDA; }

tridi_status tridi_device_status(unsigned* bits, int reset) {
  if (!bits) return TRIDI_ERROR_INVALID_VALUE;
  const DeviceInfo* d = current_device();
  if (!d) return TRIDI_ERROR_CUDA;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_status(e);
  if ((e = cudaMemcpy(bits, d->status, sizeof(unsigned), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_status(e);
  if (reset && (e = cudaMemset(d->status, 0, sizeof(unsigned))) != cudaSuccess) return cuda_status(e);
  return TRIDI_SUCCESS;
}

}  // extern "C"

// Algorithm dispatch of the host-pointer drop-ins onto the device-pointer C
// ABI, and the scratch each algorithm needs.
#include "runtime.h"
#include "tridi.h"
#include "tridi_dropin.h"

namespace tridi {

namespace {
template <class T>
struct Abi;
template <>
struct Abi<float> {
  static constexpr auto cr = tridi_cr_f32;
  static constexpr auto pcr = tridi_pcr_f32;
  static constexpr auto crpcr = tridi_crpcr_f32;
  static constexpr auto cr_nbc = tridi_cr_nbc_f32;
  static constexpr auto crpcr_nbc = tridi_crpcr_nbc_f32;
  static constexpr auto pcr_thomas = tridi_pcr_thomas_f32;
  static constexpr auto solve = tridi_solve_f32;
};
template <>
struct Abi<double> {
  static constexpr auto cr = tridi_cr_f64;
  static constexpr auto pcr = tridi_pcr_f64;
  static constexpr auto crpcr = tridi_crpcr_f64;
  static constexpr auto cr_nbc = tridi_cr_nbc_f64;
  static constexpr auto crpcr_nbc = tridi_crpcr_nbc_f64;
  static constexpr auto pcr_thomas = tridi_pcr_thomas_f64;
  static constexpr auto solve = tridi_solve_f64;
};
}  // namespace

template <class T>
size_t large_workspace_bytes(long n, long m, int layout);
template <class T>
tridi_status large_solve_device(const T* a, const T* b, const T* c, const T* d, T* x, long n, long m, int layout,
                                void* ws, size_t ws_bytes, tridi_stream_t stream);

namespace {
// pcrGaussWrapper's device path for a system size n:
//   n <= 4096                      PCR-then-Thomas (pcr_thomas.cu)
//   n <= partition_max_rows<T>()   the one-pass partition solver (partition.cu)
//   larger                         the large-system solver in the contiguous
//                                  layout (large.cu), which needs a workspace.
// The reference takes every n > MINSYSTEM = 1024 down its global-memory PCR
// path (pcrGauss_app.cu:196-228, :102-162), whatever the size.
template <class T>
bool pcr_gauss_uses_large(int n) {
  return n > partition_max_rows<T>();
}
}  // namespace

template <class T>
size_t algo_scratch_bytes(int algo, int n, int m, int param) {
  (void)param;
  if (algo == TRIDI_DROPIN_PCR_THOMAS && pcr_gauss_uses_large<T>(n) && m > 0)
    return large_workspace_bytes<T>(n, m, TRIDI_LAYOUT_CONTIGUOUS);
  return 0;
}

template <class T>
tridi_status dropin_device_solve(int algo, const T* a, const T* b, const T* c, const T* d, T* x, int n, int m,
                                 int param, void* ws, size_t ws_bytes, cudaStream_t s) {
  tridi_stream_t st = reinterpret_cast<tridi_stream_t>(s);
  switch (algo) {
    case TRIDI_DROPIN_CR: return Abi<T>::cr(a, b, c, d, x, n, m, st);
    case TRIDI_DROPIN_PCR: return Abi<T>::pcr(a, b, c, d, x, n, m, st);
    case TRIDI_DROPIN_CRPCR: return Abi<T>::crpcr(a, b, c, d, x, n, m, param, st);
    case TRIDI_DROPIN_CR_NBC:
    case TRIDI_DROPIN_CR_NBC32: return Abi<T>::cr_nbc(a, b, c, d, x, n, m, st);
    case TRIDI_DROPIN_CRPCR_NBC: return Abi<T>::crpcr_nbc(a, b, c, d, x, n, m, param, st);
    case TRIDI_DROPIN_PCR_THOMAS:
      if (n <= 4096) return Abi<T>::pcr_thomas(a, b, c, d, x, n, m, param, st);
      if (!pcr_gauss_uses_large<T>(n)) return Abi<T>::solve(a, b, c, d, x, n, m, st);
      return large_solve_device<T>(a, b, c, d, x, n, m, TRIDI_LAYOUT_CONTIGUOUS, ws, ws_bytes, st);
    default: return TRIDI_ERROR_INVALID_VALUE;
  }
}

template size_t algo_scratch_bytes<float>(int, int, int, int);
template size_t algo_scratch_bytes<double>(int, int, int, int);
template tridi_status dropin_device_solve<float>(int, const float*, const float*, const float*, const float*,
                                                 float*, int, int, int, void*, size_t, cudaStream_t);
template tridi_status dropin_device_solve<double>(int, const double*, const double*, const double*,
                                                  const double*, double*, int, int, int, void*, size_t,
                                                  cudaStream_t);

}  // namespace tridi

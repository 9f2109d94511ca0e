/* Project-written stand-in for the old NVIDIA SDK "cutil" helper header, which
   the reference's common.h includes but which no current CUDA ships.  It
   provides only the handful of macros and timer calls the reference uses, so
   that the reference sources compile unmodified for the oracle build
   (oracle/Makefile).  Timers are host wall-clock (std::chrono). */
#ifndef TRIDI_REF_SHIM_CUTIL_H
#define TRIDI_REF_SHIM_CUTIL_H
#include <stdio.h>
#include <stdlib.h>
#ifdef __cplusplus
#include <chrono>
#include <map>
#endif
#ifdef __CUDACC__
#include <cuda_runtime.h>
/* cudaThreadSynchronize was removed from the CUDA 13 headers. */
#define cudaThreadSynchronize cudaDeviceSynchronize
#define CUDA_SAFE_CALL(call)                                                    \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_),       \
              __FILE__, __LINE__);                                              \
      exit(1);                                                                  \
    }                                                                           \
  } while (0)
#else
#define CUDA_SAFE_CALL(call) (call)
#endif
#define CUT_SAFE_CALL(call) (call)
#define CUT_DEVICE_INIT(argc, argv) ((void)(argc), (void)(argv))
#ifdef __cplusplus
namespace tridi_ref_shim {
struct Timer { double acc = 0; bool on = false; std::chrono::steady_clock::time_point t0; };
static inline std::map<unsigned, Timer> &timers() { static std::map<unsigned, Timer> t; return t; }
}  // namespace tridi_ref_shim
static inline int cutCreateTimer(unsigned *id) {
  static unsigned next = 1; *id = next++; tridi_ref_shim::timers()[*id] = {}; return 1;
}
static inline int cutStartTimer(unsigned id) {
  auto &t = tridi_ref_shim::timers()[id]; t.on = true; t.t0 = std::chrono::steady_clock::now(); return 1;
}
static inline int cutStopTimer(unsigned id) {
  auto &t = tridi_ref_shim::timers()[id];
  if (t.on) t.acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t.t0).count();
  t.on = false; return 1;
}
static inline int cutResetTimer(unsigned id) { tridi_ref_shim::timers()[id] = {}; return 1; }
static inline float cutGetTimerValue(unsigned id) { return (float)tridi_ref_shim::timers()[id].acc; }
#endif
#endif

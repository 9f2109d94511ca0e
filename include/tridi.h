/*
 * tridi.h -- C ABI of the GB300-native batched tridiagonal solvers.
 *
 * Every entry point here is extern "C", takes plain pointers and sizes, and is
 * what a foreign-function binding (ctypes, cgo, JNI, ...) or the C++ drop-in
 * launchers of tridi_dropin.h call.  System i of a batch is
 *
 *     a[k] x[k-1] + b[k] x[k] + c[k] x[k+1] = d[k],   k = 0 .. n-1,
 *
 * with a[0] and c[n-1] ignored as zero (the reference assumes a[0] = c[n-1] =
 * 0).  Unless stated otherwise the layout is contiguous per system: element k
 * of system s is at s*n + k, as in every reference kernel (cr_kernel.cu:26).
 *
 * Conventions of the device-pointer API (tridi_*_f32 / _f64):
 *   - a, b, c, d, x are DEVICE pointers, 16-byte aligned (cudaMalloc memory
 *     is); a, b, c, d are read only (the reference kernels overwrite them);
 *     x receives the solution and must not alias the inputs.
 *   - Calls are asynchronous on `stream` (a cudaStream_t / CUstream; NULL is
 *     the legacy default stream) and allocate nothing, except that the first
 *     call on a device allocates that device's 64-byte status word; call
 *     tridi_init() first to do that outside of stream capture.
 *   - Status codes are returned instead of the reference's print-and-exit
 *     (CUDA_SAFE_CALL).  A bounded device-side wait that runs out is not seen
 *     by the call that launched it; tridi_device_status() reports it.
 */
#ifndef TRIDI_H
#define TRIDI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tridi_status {
  TRIDI_SUCCESS = 0,
  TRIDI_ERROR_INVALID_VALUE = 1,     /* null pointer, negative or zero count, bad enum */
  TRIDI_ERROR_UNSUPPORTED_SIZE = 2,  /* system size outside the solver's range */
  TRIDI_ERROR_MISALIGNED = 3,        /* a pointer is not 16-byte aligned */
  TRIDI_ERROR_CUDA = 4,              /* a CUDA call failed: tridi_last_cuda_error() */
  TRIDI_ERROR_DEVICE_TIMEOUT = 5,    /* a bounded device wait ran out */
  TRIDI_ERROR_NOT_CONVERGED = 6,     /* iterative refinement hit its sweep limit */
  TRIDI_ERROR_OUT_OF_MEMORY = 7,     /* admission or allocation refused */
  TRIDI_ERROR_WORKSPACE_TOO_SMALL = 8,
  TRIDI_ERROR_BUSY = 9               /* a bounded host-side queue is full */
} tridi_status;

/* Bits of the per-device status word (tridi_device_status). */
#define TRIDI_DEVERR_WAIT_TIMEOUT 0x1u /* an mbarrier / flag wait exceeded its limit */
#define TRIDI_DEVERR_BAD_PLAN 0x2u     /* a ragged work list out of the order the kernel expects */

typedef void *tridi_stream_t; /* cudaStream_t */

/* ---- library ------------------------------------------------------------ */
const char *tridi_version(void);
const char *tridi_status_string(tridi_status s);
/* The cudaError_t of the last TRIDI_ERROR_CUDA on this thread (0 if none). */
int tridi_last_cuda_error(void);
/* Allocates the current device's status word (done lazily otherwise). */
tridi_status tridi_init(void);
/* Synchronises the device, returns the OR of all TRIDI_DEVERR_* bits raised on
   the current device since the last reset, and clears them when reset != 0. */
tridi_status tridi_device_status(unsigned *bits, int reset);

/* Launch-shape tunables (process-wide; 0 = automatic).  Used by the
   autotuner and by experiments; they change speed, and at most the rounding
   of results (TRIDI_TUNE_PCR_KERNEL, TRIDI_TUNE_RESIDUAL), never the
   algorithm. */
#define TRIDI_TUNE_STAGES 1     /* cp.async.bulk pipeline stages per CTA (1..8) */
#define TRIDI_TUNE_CRPCR_REST 2 /* switch level of the CR-PCR correction solves */
#define TRIDI_TUNE_CR_ROWS 3    /* rows per thread of the CR/PCR/CR-PCR kernels (2, 4, 8, 16) */
#define TRIDI_TUNE_RESIDUAL 4   /* arithmetic of the refinements' residual and update: */
#define TRIDI_RESIDUAL_DF 1     /*   double-float (pairs of FP32, 48-bit significand; the default) */
#define TRIDI_RESIDUAL_FP64 2   /*   native FP64 */
#define TRIDI_TUNE_SERVER_COPY 5  /* host<->device transfer of servers created afterwards: */
#define TRIDI_SERVER_COPY_MEMCPY 1 /*   0 or 1 = cudaMemcpyAsync on the callers' arrays; */
#define TRIDI_SERVER_COPY_DIRECT 2 /*   2 = kernels read / write the callers' arrays (pageable memory access); */
#define TRIDI_SERVER_COPY_STAGED 3 /*   3 = pinned double-buffered staging filled by host threads */
#define TRIDI_TUNE_LARGE_TMA 6    /* interleaved FP32 large systems: 0/1 = TMA-tiled passes where they apply, 2 = off */
#define TRIDI_TUNE_WARP_STREAMS 7 /* CR/PCR/CR-PCR with a system per warp or less: 0/1 = every warp streams its own
                                     systems (no producer warp), 2 = CTA ring filled by a producer warp */
#define TRIDI_TUNE_NBC_KERNEL 8   /* bank-conflict-free CR: 0/1 = the register kernel where it has the shape
                                     (same arithmetic and results, about twice as fast), 2 = the
                                     shared-memory kernel always */
#define TRIDI_TUNE_DROPIN_CHUNK 9 /* host-pointer launchers: KiB of each coefficient array per pipelined chunk
                                     (0 = 8192 from pinned memory, 65536 from pageable memory) */
#define TRIDI_TUNE_PCR_KERNEL 10  /* FP32 PCR on 64..1024 unknowns: 0/1 = the two-phase kernel (rows transposed
                                     once between the register phases) with paired FP32 instructions,
                                     3 = the same on single rows, 2 = the hybrid warp kernel (the same
                                     algorithm throughout; results differ in rounding only) */
#define TRIDI_TUNE_DROPIN_MAPPED 11 /* host-pointer launchers (cr, pcr, crpcr, crNBC, crNBC32, crpcrNBC):
                                     0/1 = arrays that are pinned and mapped into the device's address
                                     space, or ordinary pageable arrays on a device that reaches them
                                     through the host's page tables, are read and written in place by
                                     the solver (no staging copies), 2 = always staged through device
                                     memory, 3 = in place for pinned arrays only */
#define TRIDI_TUNE_RAGGED_ORDER 12  /* plain ragged plans created afterwards: 0/1 = team items in rounds interleaved
                                     from the largest and the smallest, 2 = largest first throughout (refinement
                                     plans are always largest first) */
tridi_status tridi_set_tunable(int key, int value);
int tridi_get_tunable(int key);

/* ---- the reference's solvers, device pointers ---------------------------- */
/* Cyclic reduction.  Replaces cr() of cr_app.cu:4 / crKernel (cr_kernel.cu:1).
   n a power of two, 2 <= n <= 8192. */
tridi_status tridi_cr_f32(const float *a, const float *b, const float *c, const float *d, float *x, int n,
                          int num_systems, tridi_stream_t stream);
tridi_status tridi_cr_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                          int n, int num_systems, tridi_stream_t stream);

/* Parallel cyclic reduction.  Replaces pcr() of pcr_app.cu:5 / pcrKernel
   (pcr_kernel.cu:1).  n a power of two, 2 <= n <= 4096. */
tridi_status tridi_pcr_f32(const float *a, const float *b, const float *c, const float *d, float *x, int n,
                           int num_systems, tridi_stream_t stream);
tridi_status tridi_pcr_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                           int n, int num_systems, tridi_stream_t stream);

/* Hybrid CR -> PCR -> CR with switch level `rest_system_size` (the size of the
   intermediate system solved by PCR: a power of two, 2 <= rest <= n/2).
   Replaces crpcr() of crpcr_app.cu:5 / crpcrKernel (crpcr_kernel.cu:1). */
tridi_status tridi_crpcr_f32(const float *a, const float *b, const float *c, const float *d, float *x, int n,
                             int num_systems, int rest_system_size, tridi_stream_t stream);
tridi_status tridi_crpcr_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                             int n, int num_systems, int rest_system_size, tridi_stream_t stream);

/* Bank-conflict-free cyclic reduction.  Replaces crNBC() (crNBC.cu:123 /
   crNBCKernel :20) and crNBC32() (crNBC32banks.cu:123 / crNBC32Kernel :20).
   n a power of two, 2 <= n <= 4096 (FP64: 2048).  Two kernels with the same
   arithmetic and bit-identical results: the register CR of tridi_cr_* (rows
   in registers, the staging ring read with conflict-free 16-byte loads; used
   by default) and a shared-memory CR whose every level is conflict-free by
   construction (each level compacted into a dense array; the last 32-row
   levels in registers), selected with TRIDI_TUNE_NBC_KERNEL = 2. */
tridi_status tridi_cr_nbc_f32(const float *a, const float *b, const float *c, const float *d, float *x, int n,
                              int num_systems, tridi_stream_t stream);
tridi_status tridi_cr_nbc_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                              int n, int num_systems, tridi_stream_t stream);

/* Hybrid with the bank-conflict-free CR part.  Replaces crpcrNBC()
   (crNBC.cu:344 / crpcrNBCKernel :189).  Kernel choice as for tridi_cr_nbc_*:
   the register CR-PCR of tridi_crpcr_* by default, the shared-memory one with
   TRIDI_TUNE_NBC_KERNEL = 2. */
tridi_status tridi_crpcr_nbc_f32(const float *a, const float *b, const float *c, const float *d, float *x,
                                 int n, int num_systems, int rest_system_size, tridi_stream_t stream);
tridi_status tridi_crpcr_nbc_f64(const double *a, const double *b, const double *c, const double *d,
                                 double *x, int n, int num_systems, int rest_system_size,
                                 tridi_stream_t stream);

/* PCR-then-Thomas.  Replaces the device work of pcrGaussWrapper()
   (pcrGauss_app.cu:164; kernels pcrKernelBranchFree + serial<T,g>,
   pcrGauss_kernel.cu:1-126).  `gaussian` = g, the number of interleaved
   subsystems (a power of two, 1 <= g <= n) solved by Thomas after log2(g) PCR
   steps.  Exact for every g (the reference's step table is exact only when
   g = 2^it).  gaussian = 0: the autotuned g for n (TRIDI_AUTOTUNE_PCR_THOMAS_SPLIT),
   else n/2 for power-of-two n (else one chain per thread of the system).
   g >= n/2 on power-of-two n runs the register PCR kernels (log2(n/2) PCR
   steps leave exactly the 2-row chains PCR closes with).  Any 1 <= n <= 4096. */
tridi_status tridi_pcr_thomas_f32(const float *a, const float *b, const float *c, const float *d, float *x, int n,
                                  int num_systems, int gaussian, tridi_stream_t stream);
tridi_status tridi_pcr_thomas_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                                  int n, int num_systems, int gaussian, tridi_stream_t stream);

/* ---- GB300 additions (no counterpart kernel in the reference) ----------- */
/* Generic batched solve, any size 1 <= n <= 8704 (FP64: <= 4608), not only
   powers of two:
   partition method (per-lane Thomas-like chunk elimination in registers,
   PCR on the separator system, back substitution).  Uniform n, contiguous.
   Checked against the gold Thomas solver of tridiagonal_gold.h:26-44. */
tridi_status tridi_solve_f32(const float *a, const float *b, const float *c, const float *d, float *x, int n,
                             int num_systems, tridi_stream_t stream);
tridi_status tridi_solve_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                             int n, int num_systems, tridi_stream_t stream);

/* Large systems, any n, in either layout: TRIDI_LAYOUT_CONTIGUOUS (s*n + i) or TRIDI_LAYOUT_INTERLEAVED
   (i*num_systems + s, system-fastest).  Three kernels on `stream`: chunk
   elimination, separator-system solve, chunk back substitution.  Needs a
   device workspace of tridi_large_workspace_bytes() bytes (no allocation
   inside the call). */
#define TRIDI_LAYOUT_CONTIGUOUS 0
#define TRIDI_LAYOUT_INTERLEAVED 1
size_t tridi_large_workspace_bytes(long n, long num_systems, int elem_size);
tridi_status tridi_solve_large_f32(const float *a, const float *b, const float *c, const float *d, float *x, long n,
                                   long num_systems, int layout, void *workspace, size_t workspace_bytes,
                                   tridi_stream_t stream);
tridi_status tridi_solve_large_f64(const double *a, const double *b, const double *c, const double *d, double *x,
                                   long n, long num_systems, int layout, void *workspace, size_t workspace_bytes,
                                   tridi_stream_t stream);

/* Autotuner (GB300 addition).  Times the candidates of one tuning decision on
   a seeded synthetic batch of about sample_unknowns unknowns (<= 0: 2^24) on
   `stream`, records the fastest in the process-wide table and returns it in
   *chosen (and its time per launch in *best_ms; either may be NULL):
     TRIDI_AUTOTUNE_CRPCR_REST    key n (power of two, 4..4096): the CR-to-PCR
        switch level (rest system size, 2..n/2) that the refinement's FP32
        correction solves use; diagonally dominant systems.
     TRIDI_AUTOTUNE_PCR_THOMAS_SPLIT  key n (power of two, 2..4096): the number
        of Thomas chains g (PCR steps = log2 g) that tridi_pcr_thomas_* use
        when called with gaussian = 0; diagonally dominant systems.
     TRIDI_AUTOTUNE_RAGGED_THREADS    key: any size in the bucket
        [2^k, 2^(k+1)), k = 0..14: threads per system (32, 160 or 480) that
        ragged plans created afterwards give systems of that bucket; ADI
        systems.
     TRIDI_AUTOTUNE_CR_ROWS           key n (power of two, 32..4096): rows per
        thread (4, 8 or 16; threads per system = n / rows) of the FP32
        cr / pcr / crpcr kernels; diagonally dominant systems, timed on cr.
     TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS  as TRIDI_AUTOTUNE_RAGGED_THREADS,
        timed on the fused one-correction refinement instead of the plain
        solve, for plans created afterwards by tridi_ragged_plan_create_refine
        (the refinement issues ~3x the instructions per row of the plain
        solve, so its best group width per size can differ).
   tridi_tuned / tridi_set_tuned read and write the table (key as above,
   0 = not tuned: the built-in choice applies), tridi_autotune_reset clears
   it.  Synchronises `stream`; allocates and frees its own sample. */
#define TRIDI_AUTOTUNE_CRPCR_REST 0
#define TRIDI_AUTOTUNE_PCR_THOMAS_SPLIT 1
#define TRIDI_AUTOTUNE_RAGGED_THREADS 2
#define TRIDI_AUTOTUNE_CR_ROWS 3
#define TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS 4
tridi_status tridi_autotune(int table, long key, long sample_unknowns, tridi_stream_t stream, int *chosen,
                            float *best_ms);
int tridi_tuned(int table, long key);
tridi_status tridi_set_tuned(int table, long key, int value);
tridi_status tridi_autotune_reset(void);

/* Ragged batches (GB300 addition): systems of different sizes, concatenated --
   system s owns rows [offsets[s], offsets[s+1]) -- solved by one persistent
   launch driven by a size-bucketed work queue.  Sizes 1 .. 24480.  The plan is
   built once on the host from the offsets (host array of num_systems + 1
   entries) and uploaded to a device buffer; solves then replay it (and can be
   captured in a CUDA graph: the work counter is reset inside the call).
   a, b, c, d, x: device, 16-byte aligned, at least round_up(total_rows, 4)
   elements each. */
tridi_status tridi_ragged_plan_create(const long *offsets, int num_systems, void **plan);
/* The same for a batch that will be refined (tridi_ragged_refine_f32): threads
   per system from the TRIDI_AUTOTUNE_RAGGED_REFINE_THREADS table where tuned,
   else as tridi_ragged_plan_create.  Either kind of plan serves both calls. */
tridi_status tridi_ragged_plan_create_refine(const long *offsets, int num_systems, void **plan);
size_t tridi_ragged_plan_device_bytes(const void *plan);
int tridi_ragged_plan_items(const void *plan);
long tridi_ragged_plan_total_rows(const void *plan);
int tridi_ragged_plan_num_systems(const void *plan);
tridi_status tridi_ragged_plan_upload(const void *plan, void *dev_plan, size_t dev_plan_bytes, tridi_stream_t stream);
tridi_status tridi_ragged_plan_destroy(void *plan);
tridi_status tridi_ragged_solve_f32(const float *a, const float *b, const float *c, const float *d, float *x,
                                    const void *plan, void *dev_plan, tridi_stream_t stream);
/* Fused mixed-precision refinement of a ragged batch in one launch: per
   system, an FP32 solve, then `sweeps` times { r = d - T x and x += e in
   extended precision (TRIDI_TUNE_RESIDUAL), FP32 solve of T e = r }, all
   inside the SM; x written once in FP64 (round_up(total_rows, 4) elements).
   *dev_rel (device) receives the maximum over systems of ||d - T x||_2 /
   ||d||_2.  No host synchronisation (capturable in a CUDA graph).
   offsets_dev may be NULL. */
size_t tridi_ragged_refine_workspace_bytes(long total_rows, long num_systems);
tridi_status tridi_ragged_refine_f32(const float *a, const float *b, const float *c, const float *d, double *x,
                                     const void *plan, void *dev_plan, const long *offsets_dev, int sweeps,
                                     void *workspace, size_t workspace_bytes, double *dev_rel,
                                     tridi_stream_t stream);

/* Serving loop with continuous batching (GB300 addition).  Requests are small
   ragged batches of host arrays (FP32 a, b, c, d; FP64 x out; offsets of
   num_systems + 1 rows starting at 0); they are admitted in arrival order by
   their HBM footprint (tridi_server_request_footprint) against
   hbm_budget_bytes, coalesced into ragged batches of at most max_batch_rows
   rows, and solved with `sweeps` FP64-residual corrections (more, up to
   max_sweeps, while a batch misses its tightest tolerance) on up to
   max_inflight concurrent streams.  The caller keeps a request's arrays
   alive until tridi_server_wait returns for it. */
tridi_status tridi_server_create(size_t hbm_budget_bytes, long max_batch_rows, int max_inflight, int sweeps,
                                 int max_sweeps, void **server);
size_t tridi_server_request_footprint(long rows, long num_systems);
tridi_status tridi_server_submit(void *server, const float *a, const float *b, const float *c, const float *d,
                                 double *x, const long *offsets, int num_systems, double tol, long long *id);
/* Waits (timeout_ms < 0: forever) for request `id`; TRIDI_ERROR_BUSY on timeout.
   *status is the request's own result (TRIDI_SUCCESS, TRIDI_ERROR_NOT_CONVERGED, ...). */
tridi_status tridi_server_wait(void *server, long long id, int timeout_ms, int *status, int *sweeps,
                               double *rel_residual, double *latency_us);
tridi_status tridi_server_stats(void *server, long long *completed, long long *batches, long long *rows,
                                double *max_inflight_seen);
/* Host microseconds the slot workers spent per phase, summed over batches:
   [0] plan build, [1] allocation and host->device copies, [2] refinement up to
   the residual read-back, [3] device->host copies, [4] release. */
tridi_status tridi_server_phase_times(void *server, double *us, int n);
tridi_status tridi_server_destroy(void *server);

/* Mixed-precision iterative refinement: FP32 a, b, c, d in, FP64 x out.
   Only the residual r = d - T x and the accumulation x += e run in extended
   precision (TRIDI_TUNE_RESIDUAL: double-float by default, native FP64);
   every solve (the first and each correction) is an FP32 solve: CR-PCR for
   power-of-two contiguous n <= 4096, the partition solver for other
   contiguous n <= 8704, the large-system solver otherwise.  Stops when
   max over systems of ||d - T x|| / ||d|| <= tol, or after max_sweeps
   corrections (then returns TRIDI_ERROR_NOT_CONVERGED; x is still the best
   iterate).  *sweeps receives the number of corrections applied and
   *rel_residual the final maximum relative residual (either may be NULL).
   Synchronises `stream` once per sweep to read the residual. */
size_t tridi_refine_workspace_bytes(long n, long num_systems, int layout);
tridi_status tridi_refine_f32(const float *a, const float *b, const float *c, const float *d, double *x, long n,
                              long num_systems, int layout, double tol, int max_sweeps, void *workspace,
                              size_t workspace_bytes, tridi_stream_t stream, int *sweeps, double *rel_residual);

/* Self-check: out[i] = the FP64 value nearest hi[i] + lo[i] for normalised
   double-float pairs (|lo| <= ulp_float(hi) / 2), computed the way the fused
   refinement writes its FP64 solution (device arrays of n elements). */
tridi_status tridi_selfcheck_df_to_double(const float *hi, const float *lo, double *out, long n,
                                          tridi_stream_t stream);

/* Self-check of the bounded device waits (no counterpart in the reference):
   one CTA of num_threads threads (1..1024) waits on an mbarrier for at most
   limit_cycles SM cycles (1 .. ~2e9, the kernels' own limit).  With
   arrive != 0 the barrier completes and every wait succeeds; with arrive = 0
   nothing arrives, every wait runs out, sets TRIDI_DEVERR_WAIT_TIMEOUT in the
   device status word (tridi_device_status) and returns.  timed_out (device,
   num_threads ints) receives 1 for each thread whose wait ran out, else 0.
   Asynchronous on `stream`; faults and hangs nothing. */
tridi_status tridi_selfcheck_wait(long long limit_cycles, int arrive, int *timed_out, int num_threads,
                                  tridi_stream_t stream);

/* Allocation-free solve (no counterpart in the reference): for callers that
   cannot call cudaMalloc at solve time, e.g. an application whose device
   memory is all owned by its own pool, or a latency-critical loop that must
   not pay an allocation's implicit synchronisation.  Interleaved layout
   (element i of system s at i*num_systems + s), one thread per system runs
   the Thomas recurrence; its forward-sweep coefficients live in a 16 MiB
   array compiled into the library, so n * num_systems must not exceed
   tridi_noalloc_max_unknowns() (2^21); larger requests return
   TRIDI_ERROR_WORKSPACE_TOO_SMALL.  The array is shared by all calls on a
   device: calls that overlap on the GPU race on it.  The first call on a
   device looks up the array's address; make it before any stream capture.
   The address is kept for the life of the process: after a device reset
   (cudaDeviceReset, which unloads the library's module) it is stale, so do
   not call this entry point again in a process that reset the device.
   CUDA errors are reported by tridi_noalloc_last_cuda_error(). */
long tridi_noalloc_max_unknowns(void);
int tridi_noalloc_last_cuda_error(void);
tridi_status tridi_solve_interleaved_noalloc_f32(const float *a, const float *b, const float *c, const float *d,
                                                 float *x, long n, long num_systems, tridi_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* TRIDI_H */

/*
 * tridi_dropin.h -- the reference's host launchers, re-implemented on the
 * GB300 kernels, with the reference's exact names and signatures.
 *
 * The reference (zhangyaobit/tridiagonalsolvers) declares its launchers only
 * as bare C++ prototypes in its driver (test_tridiagonal.cpp:17-24), with
 * T = float, or double under USE_DOUBLE (common.h:8-12).  This library
 * exports both precisions as C++ overloads, so a reference driver built with
 * either T links against it unchanged:
 *
 *   void cr      (T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems);                      cr_app.cu:4
 *   void pcr     (T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems);                      pcr_app.cu:5
 *   void crpcr   (T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems,int restSystemSize);   crpcr_app.cu:5
 *   void crNBC   (T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems);                      crNBC.cu:123
 *   void crpcrNBC(T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems,int restSystemSize);   crNBC.cu:344
 *   void crNBC32 (T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems);                      crNBC32banks.cu:123
 *   void pcrGaussWrapper(T*a,T*b,T*c,T*d,T*x,int systemSize,int numSystems,int gaussian);  pcrGauss_app.cu:164
 *
 * Semantics kept from the reference: HOST pointers, contiguous layout
 * (system s, row i at s*systemSize + i), a..d are not modified, x receives
 * the solution, the call is synchronous, device 0 (the current device).
 * On a CUDA error the launcher prints the error and exits, as the
 * reference's CUDA_SAFE_CALL does (set TRIDI_DROPIN_NO_EXIT=1 to print and
 * return instead).  The reference's printed "GPU kernel time" line (after
 * numIterations = 50 timed launches, common.h:14) is produced only when
 * TRIDI_DROPIN_TIMING=1, in the reference's format.
 *
 * What changed underneath: no cudaMalloc/cudaFree per call (a persistent
 * device workspace that grows on demand, guarded by a mutex), and the batch is
 * split into chunks whose host->device copy, solve and device->host copy
 * overlap on three streams.  Arrays that are pinned and mapped into the
 * device's address space (cudaHostAlloc, cudaHostRegister with mapping) are
 * instead read and written in place by the solver over the host link, without
 * staging copies (all launchers but pcrGaussWrapper; TRIDI_TUNE_DROPIN_MAPPED
 * in tridi.h turns it off).  The solver kernels themselves are in tridi.h.
 *
 * pcrGaussWrapper takes any systemSize >= 1, as the reference's does (its
 * large path, pcrGauss_app.cu:196-228, takes every size above MINSYSTEM =
 * 1024): PCR-then-Thomas with `gaussian` chains up to 4096 rows, the one-pass
 * partition solver up to 8704 rows (FP32) / 4608 (FP64), the large-system
 * solver beyond (its workspace is part of the persistent one).  Every path
 * is exact; above 4096 rows `gaussian` does not change the result.
 *
 * The extern "C" functions below are the same launchers for foreign-function
 * callers (ctypes, cgo, JNI): status codes instead of exiting.
 */
#ifndef TRIDI_DROPIN_H
#define TRIDI_DROPIN_H

#include "tridi.h"

#ifdef __cplusplus
void cr(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems);
void cr(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems);
void pcr(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems);
void pcr(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems);
void crpcr(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems, int restSystemSize);
void crpcr(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems,
           int restSystemSize);
void crNBC(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems);
void crNBC(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems);
void crpcrNBC(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems,
              int restSystemSize);
void crpcrNBC(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems,
              int restSystemSize);
void crNBC32(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems);
void crNBC32(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems);
void pcrGaussWrapper(float *a, float *b, float *c, float *d, float *x, int systemSize, int numSystems,
                     int gaussian);
void pcrGaussWrapper(double *a, double *b, double *c, double *d, double *x, int systemSize, int numSystems,
                     int gaussian);
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Solver selector of the host-pointer API. */
typedef enum tridi_dropin_algo {
  TRIDI_DROPIN_CR = 0,        /* cr()       cr_app.cu:4 */
  TRIDI_DROPIN_PCR = 1,       /* pcr()      pcr_app.cu:5 */
  TRIDI_DROPIN_CRPCR = 2,     /* crpcr()    crpcr_app.cu:5, param = restSystemSize */
  TRIDI_DROPIN_CR_NBC = 3,    /* crNBC()    crNBC.cu:123 */
  TRIDI_DROPIN_CRPCR_NBC = 4, /* crpcrNBC() crNBC.cu:344, param = restSystemSize */
  TRIDI_DROPIN_CR_NBC32 = 5,  /* crNBC32()  crNBC32banks.cu:123 */
  TRIDI_DROPIN_PCR_THOMAS = 6 /* pcrGaussWrapper() pcrGauss_app.cu:164, param = gaussian */
} tridi_dropin_algo;

/* Host-pointer launchers: copy in, solve, copy out, synchronous.  `param` is
   restSystemSize or gaussian where the algorithm takes one (else ignored). */
tridi_status tridi_dropin_solve_f32(int algo, const float *a, const float *b, const float *c, const float *d,
                                    float *x, int system_size, int num_systems, int param);
tridi_status tridi_dropin_solve_f64(int algo, const double *a, const double *b, const double *c,
                                    const double *d, double *x, int system_size, int num_systems, int param);
/* 1 when the current device reads and writes ordinary pageable host memory
   through the host's own page tables (Grace-class hosts), so the launchers
   above solve malloc'd arrays in place instead of staging them; else 0.
   (TRIDI_TUNE_DROPIN_MAPPED, tridi.h, selects the path.) */
int tridi_dropin_pageable_in_place(void);
/* Frees the persistent drop-in workspace of the current device. */
tridi_status tridi_dropin_release(void);

/* Text dump of a host solution in the reference driver's format
   (writeResultToFile, tridiagonal_gold.h:96-107; written by
   test_tridiagonal.cpp:103-104 as cpu_result.txt / gpu_result.txt): per
   system a line "***The following is the result of the equation set <s>",
   then one value per line in the C++ stream's default format (6 significant
   digits), so dumps of both builds diff line by line. */
tridi_status tridi_write_result_file_f32(const float *x, int num_systems, int system_size, const char *path);
tridi_status tridi_write_result_file_f64(const double *x, int num_systems, int system_size, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* TRIDI_DROPIN_H */

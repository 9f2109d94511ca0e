/*
 * Oracle: CPU restatement of the reference's gold Thomas solver, its test
 * generator and its comparator.  TEST INFRASTRUCTURE ONLY: the tests, the
 * smoke check and bench.py's CPU-baseline leg may call it as the checker; the
 * product path never links or calls anything in this file.
 *
 * Every function cites the reference routine it restates
 * (tridiagonalsolvers/tridiagonal_gold.h).  The arithmetic follows the
 * reference statement by statement, so that, compiled with
 * -ffp-contract=off (no fused multiply-add, identical on x86-64 and
 * aarch64), the FP32 and FP64 results are bit-identical to the reference
 * header compiled the same way.  That identity is checked by
 * tests/test_oracle.py against oracle/_ref (the reference itself, built from
 * its own sources by oracle/Makefile) and against the committed golden
 * vectors in tests/golden/.
 *
 * The T macro of the reference (common.h:8-12) becomes a _f32 / _f64 suffix.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define GOLD_DEFINE(T, SUF, FABS, SQRT)                                              \
  /* tridiagonal_gold.h:26-44 -- Thomas algorithm without pivoting.               \
     Like the reference it overwrites c and d (c[n-1] is zeroed, then c and d     \
     receive the eliminated coefficients). */                                      \
  void gold_serial_##SUF(T *a, T *b, T *c, T *d, T *x, int n) {                     \
    c[n - 1] = 0;                                                                   \
    c[0] = c[0] / b[0];                                                             \
    d[0] = d[0] / b[0];                                                             \
    for (int i = 1; i < n; i++) {                                                   \
      c[i] = c[i] / (b[i] - a[i] * c[i - 1]);                                       \
      d[i] = (d[i] - d[i - 1] * a[i]) / (b[i] - a[i] * c[i - 1]);                   \
    }                                                                               \
    x[n - 1] = d[n - 1];                                                            \
    for (int i = n - 2; i >= 0; i--) x[i] = d[i] - c[i] * x[i + 1];                 \
  }                                                                                 \
                                                                                    \
  /* tridiagonal_gold.h:47-53 -- one system after another, contiguous layout. */  \
  void gold_many_systems_##SUF(T *a, T *b, T *c, T *d, T *x, int n, int m) {        \
    for (long i = 0; i < m; i++)                                                    \
      gold_serial_##SUF(a + i * n, b + i * n, c + i * n, d + i * n, x + i * n, n);  \
  }                                                                                 \
                                                                                    \
  /* tridiagonal_gold.h:56-72 -- the reference's 4-thread split.  It keeps the    \
     reference's behaviour exactly: chunk = m/4 systems per thread, so the        \
     m % 4 trailing systems are NOT solved (their x is left untouched). */        \
  void gold_multithread_many_systems_##SUF(T *a, T *b, T *c, T *d, T *x, int n,     \
                                           int m) {                                 \
    const int nthreads = 4;                                                         \
    const int chunk = m / nthreads;                                                 \
    _Pragma("omp parallel for num_threads(4) schedule(static, 1)")                  \
    for (int me = 0; me < nthreads; me++) {                                         \
      for (long i = (long)me * chunk; i < (long)me * chunk + chunk; i++)            \
        gold_serial_##SUF(a + i * n, b + i * n, c + i * n, d + i * n, x + i * n, n); \
    }                                                                               \
  }                                                                                 \
                                                                                    \
  /* Every system, split over `nthreads` host threads (0 = all cores).  Same     \
     per-system arithmetic as gold_serial; this is the all-cores CPU baseline. */  \
  void gold_many_systems_omp_##SUF(T *a, T *b, T *c, T *d, T *x, int n, int m,      \
                                   int nthreads) {                                  \
    if (nthreads <= 0) nthreads = gold_max_threads();                               \
    _Pragma("omp parallel for num_threads(nthreads) schedule(static)")             \
    for (long i = 0; i < m; i++)                                                    \
      gold_serial_##SUF(a + i * n, b + i * n, c + i * n, d + i * n, x + i * n, n);  \
  }                                                                                 \
                                                                                    \
  /* tridiagonal_gold.h:75-78 */                                                    \
  static T rand01_##SUF(void) { return (T)rand() / (T)RAND_MAX; }                   \
                                                                                    \
  /* tridiagonal_gold.h:81-94 -- the reference's input generator (libc rand()).   \
     The caller seeds with gold_srand (the reference never seeds: seed 1). */     \
  void gold_test_generation_##SUF(T *a, T *b, T *c, T *d, T *x, int n) {            \
    for (int j = 0; j < n; j++) {                                                   \
      b[j] = 8 + rand01_##SUF();                                                    \
      a[j] = 3 + rand01_##SUF();                                                    \
      c[j] = 2 + rand01_##SUF();                                                    \
      d[j] = 5 + rand01_##SUF();                                                    \
      x[j] = 0;                                                                     \
    }                                                                               \
    a[0] = 0;                                                                       \
    c[n - 1] = 0;                                                                   \
  }                                                                                 \
                                                                                    \
  /* tridiagonal_gold.h:111-130 -- root-mean-square difference of one system. */  \
  T gold_compare_##SUF(const T *x1, const T *x2, int n) {                           \
    T root = 0;                                                                     \
    for (int i = 0; i < n; i++) root += (x1[i] - x2[i]) * (x1[i] - x2[i]);          \
    root /= n;                                                                      \
    return SQRT(root);                                                              \
  }                                                                                 \
                                                                                    \
  /* tridiagonal_gold.h:133-148 -- number of systems whose RMS difference        \
     exceeds eps or is NaN.  rms_out (may be NULL) receives each system's RMS. */  \
  int gold_compare_many_systems_##SUF(const T *x1, const T *x2, int n, int m,       \
                                      T eps, T *rms_out) {                          \
    int failed = 0;                                                                 \
    for (long i = 0; i < m; i++) {                                                  \
      T diff = gold_compare_##SUF(x1 + i * n, x2 + i * n, n);                       \
      if (rms_out) rms_out[i] = diff;                                               \
      if (diff > eps || diff != diff) failed++;                                     \
    }                                                                               \
    return failed;                                                                  \
  }

int gold_max_threads(void) {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}

void gold_srand(unsigned seed) { srand(seed); }

GOLD_DEFINE(float, f32, fabsf, sqrtf)
GOLD_DEFINE(double, f64, fabs, sqrt)

/* The strict oracle used by the parity tests: the gold Thomas solver of
   tridiagonal_gold.h:26-44 run in FP64 on FP32 inputs, without touching the
   caller's arrays.  `layout` 0 = contiguous (sys*n + i), 1 = interleaved
   (i*m + sys).  nthreads <= 0 uses every core. */
void gold_solve_f64_from_f32(const float *a, const float *b, const float *c,
                             const float *d, double *x, int n, int m, int layout,
                             int nthreads) {
  if (nthreads <= 0) nthreads = gold_max_threads();
#pragma omp parallel num_threads(nthreads)
  {
    double *buf = (double *)malloc(sizeof(double) * 5 * (size_t)n);
    double *aa = buf, *bb = buf + n, *cc = buf + 2 * (size_t)n, *dd = buf + 3 * (size_t)n,
           *xx = buf + 4 * (size_t)n;
#pragma omp for schedule(static)
    for (long s = 0; s < m; s++) {
      for (long i = 0; i < n; i++) {
        long k = layout ? i * m + s : s * n + i;
        aa[i] = a[k]; bb[i] = b[k]; cc[i] = c[k]; dd[i] = d[k];
      }
      gold_serial_f64(aa, bb, cc, dd, xx, n);
      for (long i = 0; i < n; i++) x[layout ? i * m + s : s * n + i] = xx[i];
    }
    free(buf);
  }
}

/* FP64 residual of an FP32 system at a given solution: per system,
   ||d - T x||_2 / ||d||_2 with T the tridiagonal matrix (a sub, b main, c
   super).  x is FP64; pass an FP32 solution through x32 instead (x = NULL).
   Used to state the relative residual of every result. */
void gold_rel_residual(const float *a, const float *b, const float *c, const float *d,
                       const double *x, const float *x32, int n, int m, int layout,
                       double *out, int nthreads) {
  if (nthreads <= 0) nthreads = gold_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long s = 0; s < m; s++) {
    double rr = 0, dd = 0;
    for (long i = 0; i < n; i++) {
      long k = layout ? i * m + s : s * n + i;
      long km = layout ? (i - 1) * m + s : k - 1, kp = layout ? (i + 1) * m + s : k + 1;
      double xi = x ? x[k] : (double)x32[k];
      double r = (double)d[k] - (double)b[k] * xi;
      if (i > 0) r -= (double)a[k] * (x ? x[km] : (double)x32[km]);
      if (i < n - 1) r -= (double)c[k] * (x ? x[kp] : (double)x32[kp]);
      rr += r * r;
      dd += (double)d[k] * (double)d[k];
    }
    out[s] = dd > 0 ? sqrt(rr) / sqrt(dd) : sqrt(rr);
  }
}

/* Ragged batches (test infrastructure for the ragged solver, which has no
   reference counterpart): system s owns rows [off[s], off[s+1]) of the
   concatenated arrays.  Per system, the FP64 gold Thomas solution (into x64,
   may be NULL), the relative residual of a given solution (x FP64 or x32
   FP32, one of them non-NULL) and the forward error max|x - x64| /
   max|x64| (fwd, may be NULL).  Same Thomas recurrence and residual as the
   uniform routines above (tridiagonal_gold.h:26-44). */
void gold_check_ragged(const float *a, const float *b, const float *c, const float *d,
                       const double *x, const float *x32, const long *off, int m,
                       double *x64, double *res, double *fwd, int nthreads) {
  if (nthreads <= 0) nthreads = gold_max_threads();
  long nmax = 0;
  for (int s = 0; s < m; s++)
    if (off[s + 1] - off[s] > nmax) nmax = off[s + 1] - off[s];
#pragma omp parallel num_threads(nthreads)
  {
    double *buf = (double *)malloc(sizeof(double) * 5 * (size_t)(nmax > 0 ? nmax : 1));
    double *aa = buf, *bb = buf + nmax, *cc = buf + 2 * nmax, *dd = buf + 3 * nmax, *xx = buf + 4 * nmax;
#pragma omp for schedule(dynamic, 64)
    for (long s = 0; s < m; s++) {
      const long lo = off[s], n = off[s + 1] - off[s];
      double rr = 0, dn = 0, err = 0, big = 0;
      for (long i = 0; i < n; i++) {
        const long k = lo + i;
        const double xi = x ? x[k] : (double)x32[k];
        double r = (double)d[k] - (double)b[k] * xi;
        if (i > 0) r -= (double)a[k] * (x ? x[k - 1] : (double)x32[k - 1]);
        if (i < n - 1) r -= (double)c[k] * (x ? x[k + 1] : (double)x32[k + 1]);
        rr += r * r;
        dn += (double)d[k] * (double)d[k];
        aa[i] = a[k]; bb[i] = b[k]; cc[i] = c[k]; dd[i] = d[k];
      }
      if (res) res[s] = dn > 0 ? sqrt(rr) / sqrt(dn) : sqrt(rr);
      if (n > 0 && (x64 || fwd)) {
        gold_serial_f64(aa, bb, cc, dd, xx, (int)n);
        for (long i = 0; i < n; i++) {
          const double xi = x ? x[lo + i] : (double)x32[lo + i];
          if (x64) x64[lo + i] = xx[i];
          if (fabs(xi - xx[i]) > err || xi != xi) err = xi != xi ? INFINITY : fabs(xi - xx[i]);
          if (fabs(xx[i]) > big) big = fabs(xx[i]);
        }
      }
      if (fwd) fwd[s] = big > 0 ? err / big : err;
    }
    free(buf);
  }
}

// Exposes the reference's own gold routines (tridiagonal_gold.h, compiled from
// the reference sources where they lie) under C names so that the oracle tests
// can check gold.c against the reference itself.  Built by oracle/Makefile into
// oracle/_ref/ (never committed, never shipped in the product).  Compiled twice:
// once as is (T = float) and once with -DUSE_DOUBLE (T = double), common.h:8-12.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include "tridiagonal_gold.h"

#ifdef USE_DOUBLE
#define REF_SUF(name) name##_f64
#else
#define REF_SUF(name) name##_f32
#endif

extern "C" {
void REF_SUF(ref_serial_many_systems)(T *a, T *b, T *c, T *d, T *x, int n, int m) {
  serialManySystems(a, b, c, d, x, n, m);  // tridiagonal_gold.h:47
}
void REF_SUF(ref_multithread_many_systems)(T *a, T *b, T *c, T *d, T *x, int n, int m) {
  multiThreadManySystems(a, b, c, d, x, n, m);  // tridiagonal_gold.h:56
}
void REF_SUF(ref_test_generation)(T *a, T *b, T *c, T *d, T *x, int n) {
  testGeneration(a, b, c, d, x, n);  // tridiagonal_gold.h:81
}
T REF_SUF(ref_compare)(T *x1, T *x2, int n) { return compare(x1, x2, n, 0); }  // :111
void REF_SUF(ref_srand)(unsigned s) { srand(s); }
void REF_SUF(ref_write_result_file)(T *x, int m, int n, const char *path) {
  writeResultToFile(x, m, n, const_cast<char *>(path));  // tridiagonal_gold.h:96
}
}

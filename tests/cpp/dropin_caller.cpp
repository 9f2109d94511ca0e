// A C++ caller of the reference's host launchers, declared the way the
// reference's own driver declares them (test_tridiagonal.cpp:17-26: bare
// prototypes, T = float, or double with -DUSE_DOUBLE as in common.h:8-12)
// and linked against libtridi.so.  That it links shows the library exports
// the reference's C++ symbols in this precision; running it exercises the
// C++ overloads themselves, with their exit-on-error and timing behaviour.
//
//   dropin_caller <launcher> <systemSize> <numSystems> <param> <in.bin> <out.bin> [result.txt]
//
// in.bin holds a, b, c, d (numSystems * systemSize values of T each, in that
// order); x is written to out.bin and, if given, to result.txt in the
// reference driver's text format.  param is restSystemSize (crpcr, crpcrNBC)
// or gaussian (pcrGaussWrapper) and ignored otherwise.  The line
// "returned" is printed after the launcher returns, so a caller can tell an
// exit inside the launcher from a return.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef USE_DOUBLE
#define T double
#else
#define T float
#endif

void crpcr(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems, int restSystemSize);
void crpcrNBC(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems, int restSystemSize);
void pcr(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems);
void cr(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems);
void crNBC(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems);
void crNBC32(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems);
void pcrGaussWrapper(T *a, T *b, T *c, T *d, T *x, int systemSize, int numSystems, int gaussian);

extern "C" int tridi_write_result_file_f32(const float *x, int num_systems, int system_size, const char *path);
extern "C" int tridi_write_result_file_f64(const double *x, int num_systems, int system_size, const char *path);

static int usage() {
  fprintf(stderr, "usage: dropin_caller <launcher> <n> <m> <param> <in.bin> <out.bin> [result.txt]\n");
  return 2;
}

int main(int argc, char **argv) {
  if (argc < 7) return usage();
  const char *name = argv[1];
  const int n = atoi(argv[2]), m = atoi(argv[3]), param = atoi(argv[4]);
  if (n <= 0 || m <= 0) return usage();
  const size_t count = (size_t)n * m;
  std::vector<T> buf(4 * count), x(count, T(0));
  FILE *f = fopen(argv[5], "rb");
  if (!f || fread(buf.data(), sizeof(T), buf.size(), f) != buf.size()) {
    fprintf(stderr, "cannot read %s\n", argv[5]);
    return 2;
  }
  fclose(f);
  T *a = buf.data(), *b = a + count, *c = b + count, *d = c + count;
  if (!strcmp(name, "cr")) cr(a, b, c, d, x.data(), n, m);
  else if (!strcmp(name, "pcr")) pcr(a, b, c, d, x.data(), n, m);
  else if (!strcmp(name, "crpcr")) crpcr(a, b, c, d, x.data(), n, m, param);
  else if (!strcmp(name, "crNBC")) crNBC(a, b, c, d, x.data(), n, m);
  else if (!strcmp(name, "crpcrNBC")) crpcrNBC(a, b, c, d, x.data(), n, m, param);
  else if (!strcmp(name, "crNBC32")) crNBC32(a, b, c, d, x.data(), n, m);
  else if (!strcmp(name, "pcrGaussWrapper")) pcrGaussWrapper(a, b, c, d, x.data(), n, m, param);
  else return usage();
  printf("returned\n");
  fflush(stdout);
  f = fopen(argv[6], "wb");
  if (!f || fwrite(x.data(), sizeof(T), count, f) != count) {
    fprintf(stderr, "cannot write %s\n", argv[6]);
    return 2;
  }
  fclose(f);
  if (argc > 7) {
#ifdef USE_DOUBLE
    if (tridi_write_result_file_f64(x.data(), m, n, argv[7]) != 0) return 3;
#else
    if (tridi_write_result_file_f32(x.data(), m, n, argv[7]) != 0) return 3;
#endif
  }
  return 0;
}

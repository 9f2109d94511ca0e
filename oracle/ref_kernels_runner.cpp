// Launches the reference's own GPU kernels (compiled for sm_103a from the
// reference sources into oracle/_ref/{f32,f64}/*.cubin by oracle/Makefile)
// with exactly the grid, block and dynamic shared-memory sizes that the
// reference's host launchers use.  TEST INFRASTRUCTURE ONLY: the GPU parity
// tests compare the product kernels against these, and nothing in the product
// calls this file.
//
// The launch sequences restate the reference launchers:
//   cr        cr_app.cu:37-44          grid m, block n/2, smem 5 n sizeof(T)
//   pcr       pcr_app.cu:31-40         grid m, block n,   smem 5 (n+1) sizeof(T)
//   crpcr     crpcr_app.cu:32-41       grid m, block n/2, smem (5 (n+1) + 5 rest) sizeof(T)
//   crNBC     crNBC.cu:152-161         grid m, block n/2, smem 5 n sizeof(T) 17/16
//   crpcrNBC  crNBC.cu:373-382         grid m, block n/2, smem 5 n sizeof(T) 17/16 + 5 rest sizeof(T)
//   crNBC32   crNBC32banks.cu:152-161  grid m, block n/2, smem 5 n sizeof(T) 33/32
//   pcrGauss  pcrGauss_app.cu:4-162    pcrGaussSmall (n <= 1024) or solveLargeSystem
//
// Every launch is asynchronous on the caller's stream and operates on device
// pointers that the caller owns.  Like the reference kernels, they overwrite
// their a, b, c, d inputs (pcrGauss leaves x in d or in d2).
// The one deliberate difference from the reference launchers: launches that
// need more than 48 KB of dynamic shared memory opt in with
// CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, which GT200-era code never
// had to do; it changes no arithmetic.
#include <cuda.h>

#include <cstdio>
#include <map>
#include <string>

namespace {

struct Module {
  CUmodule mod = nullptr;
};

std::map<std::string, Module> g_modules;  // key: "<prec>/<file>"
std::string g_dir;
CUcontext g_ctx = nullptr;
char g_err[512];

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  snprintf(g_err, sizeof g_err, "%s: %s", what, s ? s : "?");
  return (int)r ? (int)r : -1;
}

int ensure_ctx() {
  if (!g_ctx) {
    CUresult r = cuInit(0);
    if (r) return fail("cuInit", r);
    CUdevice dev;
    r = cuDeviceGet(&dev, 0);
    if (r) return fail("cuDeviceGet", r);
    r = cuDevicePrimaryCtxRetain(&g_ctx, dev);
    if (r) return fail("cuDevicePrimaryCtxRetain", r);
  }
  CUresult r = cuCtxSetCurrent(g_ctx);
  return r ? fail("cuCtxSetCurrent", r) : 0;
}

int get_fn(bool dbl, const char* file, const std::string& name, CUfunction* f) {
  std::string key = std::string(dbl ? "f64/" : "f32/") + file;
  auto it = g_modules.find(key);
  if (it == g_modules.end()) {
    Module m;
    std::string path = g_dir + "/" + key + ".cubin";
    CUresult r = cuModuleLoad(&m.mod, path.c_str());
    if (r) return fail(path.c_str(), r);
    it = g_modules.emplace(key, m).first;
  }
  CUresult r = cuModuleGetFunction(f, it->second.mod, name.c_str());
  return r ? fail(name.c_str(), r) : 0;
}

int launch(CUfunction f, int grid, int block, size_t smem, void* stream, void** args) {
  if (smem > 48 * 1024) {
    CUresult r = cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
    if (r) return fail("cuFuncSetAttribute", r);
  }
  CUresult r = cuLaunchKernel(f, grid, 1, 1, block, 1, 1, (unsigned)smem, (CUstream)stream, args, nullptr);
  return r ? fail("cuLaunchKernel", r) : 0;
}

// Itanium-mangled kernel names: the reference kernels have C++ linkage.
std::string tname(bool dbl) { return dbl ? "d" : "f"; }
std::string five_ptr(const char* base, bool dbl) {  // name(T*,T*,T*,T*,T*)
  return std::string(base) + "P" + tname(dbl) + "S_S_S_S_";
}

// (gaussian -> iteration) template tables of pcrGaussSmall (pcrGauss_app.cu:58-96)
// and pcrGaussLarge (pcrGauss_app.cu:12-47).
int small_it(int g) {
  switch (g) { case 1: return 0; case 2: return 1; case 4: return 2; case 8: return 3; case 16: return 3;
    case 32: return 3; case 64: return 3; case 128: return 4; case 256: return 5; case 512: return 6; }
  return -1;
}
int large_it(int g) {
  switch (g) { case 1: return 0; case 2: return 1; case 4: return 2; case 8: return 2; case 16: return 2;
    case 32: return 2; case 64: return 2; case 128: return 3; case 256: return 4; case 512: return 5; }
  return -1;
}
std::string branch_free_name(bool dbl, int g, int it, bool large) {
  return "_Z19pcrKernelBranchFreeI" + tname(dbl) + "Li1ELi" + std::to_string(g) + "ELi" +
         std::to_string(it) + "EEvPT_S1_S1_S1_ii" + (large ? "ii" : "");
}

}  // namespace

extern "C" {

const char* refk_last_error() { return g_err; }

// dir holds f32/ and f64/ sub-directories of cubins.
int refk_init(const char* dir) {
  g_dir = dir;
  return ensure_ctx();
}

// kind: 0 cr, 1 pcr, 2 crpcr, 3 crNBC, 4 crpcrNBC, 5 crNBC32
int refk_solve(int kind, int dbl, void* a, void* b, void* c, void* d, void* x, int n, int m, int rest,
               void* stream) {
  if (int e = ensure_ctx()) return e;
  const size_t ts = dbl ? 8 : 4;
  CUfunction f;
  int e = 0, block = n / 2;
  size_t smem = 0;
  void* args5[] = {&a, &b, &c, &d, &x};
  void* args6[] = {&a, &b, &c, &d, &x, &rest};
  void** args = args5;
  switch (kind) {
    case 0: e = get_fn(dbl, "cr_app", five_ptr("_Z8crKernel", dbl), &f); smem = n * 5 * ts; break;
    case 1: e = get_fn(dbl, "pcr_app", five_ptr("_Z9pcrKernel", dbl), &f); block = n; smem = (n + 1) * 5 * ts; break;
    case 2:
      e = get_fn(dbl, "crpcr_app", five_ptr("_Z11crpcrKernel", dbl) + "i", &f);
      smem = (n + 1) * 5 * ts + rest * 5 * ts; args = args6; break;
    case 3: e = get_fn(dbl, "crNBC", five_ptr("_Z11crNBCKernel", dbl), &f); smem = n * 5 * ts * 17 / 16; break;
    case 4:
      e = get_fn(dbl, "crNBC", five_ptr("_Z14crpcrNBCKernel", dbl) + "i", &f);
      smem = n * 5 * ts * 17 / 16 + rest * 5 * ts; args = args6; break;
    case 5: e = get_fn(dbl, "crNBC32banks", five_ptr("_Z13crNBC32Kernel", dbl), &f); smem = n * 5 * ts * 33 / 32; break;
    default: snprintf(g_err, sizeof g_err, "bad kind %d", kind); return -1;
  }
  if (e) return e;
  return launch(f, m, block, smem, stream, args);
}

// pcrGaussWrapper's device work (pcrGauss_app.cu:196-253) for one call: the
// small path for n <= MINSYSTEM (1024), else solveLargeSystem with the ping
// buffers a2..d2.  *x_in_second is set to 1 when the solution was left in d2
// (pcrGauss_app.cu:221-228), else it is in d.
int refk_pcr_gauss(int dbl, void* a, void* b, void* c, void* d, void* a2, void* b2, void* c2, void* d2, int n,
                   int m, int g, void* stream, int* x_in_second) {
  if (int e = ensure_ctx()) return e;
  const size_t ts = dbl ? 8 : 4;
  const int MINSYSTEM = 1024;
  CUfunction f;
  *x_in_second = 0;
  if (n <= MINSYSTEM) {  // pcrGaussSmall, pcrGauss_app.cu:49-100
    int it = small_it(g);
    if (it < 0) { snprintf(g_err, sizeof g_err, "unsupported gaussian %d", g); return -1; }
    if (int e = get_fn(dbl, "pcrGauss_app", branch_free_name(dbl, g, it, false), &f)) return e;
    int ne = m, ss = n;
    void* args[] = {&a, &b, &c, &d, &ne, &ss};
    return launch(f, m, n, (n + 1) * 5 * ts, stream, args);
  }
  // solveLargeSystem, pcrGauss_app.cu:102-162.  The globalPCROneStep loop
  // (:121-132) never runs because numSystemsSplit starts at systemSize.
  int count = 0, stride = 1, systemSize = n, numSystems = m;
  if (systemSize / stride > MINSYSTEM) {
    std::string nm = std::string("_Z23globalPCROneBlockSystemI") + tname(dbl) + "Li1024EEvPT_S1_S1_S1_S1_S1_S1_S1_ii";
    if (int e = get_fn(dbl, "pcrGauss_app", nm, &f)) return e;
    void* args[] = {&a2, &b2, &c2, &d2, &a, &b, &c, &d, &systemSize, &stride};
    if (int e = launch(f, numSystems, MINSYSTEM, 0, stream, args)) return e;
    while (systemSize > MINSYSTEM) {
      numSystems *= 2;
      systemSize /= 2;
      stride *= 2;
      count += 1;
    }
  }
  int it = large_it(g);
  if (it < 0) { snprintf(g_err, sizeof g_err, "unsupported gaussian %d", g); return -1; }
  if (int e = get_fn(dbl, "pcrGauss_app", branch_free_name(dbl, g, it, true), &f)) return e;
  void *pa = a, *pb = b, *pc = c, *pd = d;
  if (count % 2) { pa = a2; pb = b2; pc = c2; pd = d2; }
  int ne = numSystems, ss = systemSize, st = stride, bps = stride;
  void* args[] = {&pa, &pb, &pc, &pd, &ne, &ss, &st, &bps};
  if (int e = launch(f, numSystems, systemSize, (systemSize + 2) * 5 * ts, stream, args)) return e;
  *x_in_second = count % 2;
  return 0;
}

}  // extern "C"

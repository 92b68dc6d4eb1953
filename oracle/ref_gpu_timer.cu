// ref_gpu_timer.cu -- launches the reference's own CUDA kernels (cuda/src/matfun_cuda.cu of the reference, compiled
// for sm_103a into oracle/_ref/matfun_cuda_ref.cubin by oracle/Makefile.ref) on caller-provided device buffers.
// TEST AND BENCHMARK INFRASTRUCTURE ONLY: it gives the GPU bar (the reference kernel on the same GPU and inputs)
// and a second parity reference; the product never calls it.
//
// The kernels are found by name in the module (they live in an anonymous namespace, so their mangled names carry a
// module-specific prefix) and launched with the reference's launch shapes and by-value coefficient structs
// (cuda/src/matfun_cuda.cu:18-24, 51-56, 144-159): smf_eval_kernel / smf_hess_kernel with 32 threads per block and
// Coef {double c[30]}, gmf_eval_kernel with 64 threads per block and GCoef {double b[200]}.
//   nvcc -shared -Xcompiler -fPIC -o oracle/ref_gpu_timer.so oracle/ref_gpu_timer.cu -lcuda
#include <cuda.h>

#include <cstdint>
#include <cstring>
#include <string>

namespace {
CUmodule g_mod = nullptr;

struct Coef30 { double c[30]; };
struct Coef200 { double b[200]; };

CUfunction find(const std::string &pattern) {
  unsigned int count = 0;
  if (cuModuleGetFunctionCount(&count, g_mod) != CUDA_SUCCESS || count == 0) return nullptr;
  CUfunction fs[256];
  if (count > 256) count = 256;
  if (cuModuleEnumerateFunctions(fs, count, g_mod) != CUDA_SUCCESS) return nullptr;
  for (unsigned int i = 0; i < count; i++) {
    const char *name = nullptr;
    if (cuFuncGetName(&name, fs[i]) == CUDA_SUCCESS && name && std::strstr(name, pattern.c_str())) return fs[i];
  }
  return nullptr;
}

// second divided difference coefficients (smf_kernel.hpp:135-146), restated
void dd2_coef(int kind, double al, double *c) {
  if (kind == 0) {
    double f = 0.5;
    for (int k = 0; k < 30; k++) { c[k] = f; f /= (k + 3.0); }
  } else if (kind == 1) {
    for (int k = 0; k < 30; k++) c[k] = (k % 2 ? 1.0 : -1.0) / (k + 2.0);
  } else {
    double b = al * (al - 1.0) / 2.0;
    for (int k = 0; k < 30; k++) { c[k] = b; b *= (al - k - 2.0) / (k + 3.0); }
  }
}

// group-series coefficients (gmf_kernel.hpp:48-53), restated
void series_coef(int kind, double al, double *b) {
  b[0] = 1.0;
  for (int j = 1; j < 200; j++) b[j] = kind == 0 ? b[j - 1] / j : (kind == 1 ? (j % 2 ? 1.0 : -1.0) / j : b[j - 1] * (al - j + 1) / j);
}
}  // namespace

extern "C" int refgpu_load(const char *cubin) {
  if (g_mod) return 0;
  CUcontext ctx = nullptr;
  if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS || !ctx) return -1;  // the caller's (primary) context must be current
  return cuModuleLoad(&g_mod, cubin) == CUDA_SUCCESS ? 0 : -2;
}

// gmf (matrix layout): kind 0 exp, 1 log, 2 pow, 3 sqrt (-> pow 0.5); order 0, 1, 2
extern "C" int refgpu_gmf(int kind, double alpha, int order, int64_t n, const double *A, double *F, double *J,
                          double *H, void *stream) {
  if (!g_mod || n <= 0) return -1;
  if (kind == 3) kind = 2, alpha = 0.5;
  if (kind != 2) alpha = 0.0;
  const std::string pat = "gmf_eval_kernelILi" + std::to_string(kind) + "ELi" + std::to_string(order) + "E";
  CUfunction f = find(pat);
  if (!f) return -3;
  Coef200 bt;
  series_coef(kind, alpha, bt.b);
  void *params[] = {&n, &A, &F, &J, &H, &alpha, &bt};
  const unsigned blocks = (unsigned)((n + 63) / 64);
  return cuLaunchKernel(f, blocks, 1, 1, 64, 1, 1, 0, (CUstream)stream, params, nullptr) == CUDA_SUCCESS ? 0 : -2;
}

// smf, Voigt layout: order 2 -> smf_hess_kernel, else smf_eval_kernel; both 32 threads per block
extern "C" int refgpu_smf(int kind, double alpha, int order, int64_t n, const double *x, double *F, double *J,
                          double *H, void *stream) {
  if (!g_mod || n <= 0) return -1;
  if (kind != 2) alpha = kind == 3 ? 0.5 : 0.0;
  const std::string pat = std::string(order == 2 ? "smf_hess_kernelILi" : "smf_eval_kernelILi") +
                          std::to_string(kind) + "ELb0E";
  CUfunction f = find(pat);
  if (!f) return -3;
  Coef30 c2;
  dd2_coef(kind, alpha, c2.c);
  double *Jp = order >= 1 ? J : nullptr, *Hp = order >= 2 ? H : nullptr;
  void *params[] = {&n, &x, &F, &Jp, &Hp, &alpha, &c2};
  const unsigned blocks = (unsigned)((n + 31) / 32);
  return cuLaunchKernel(f, blocks, 1, 1, 32, 1, 1, 0, (CUstream)stream, params, nullptr) == CUDA_SUCCESS ? 0 : -2;
}

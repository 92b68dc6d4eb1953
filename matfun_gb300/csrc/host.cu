// host.cu -- host-buffer entry points: the reference's CPU API (smf_eval, smf_eval_matrix, gmf_eval of
// c/include/matfun/matfun.h:28-41: host arrays, synchronous, -1 / -3 return codes) evaluated on the current GPU.
//
// Page-locked host arrays (cudaHostAlloc / cudaMallocHost / registered) are mapped into the GPU's address space, and on
// GB300 the GPU reaches host memory over NVLink-C2C: when every array of a call is page-locked and mapped, the kernels
// read the inputs and write F, J, H in place, with no device buffer and no copy engine (the stores stream over the
// link while the SMs compute).  Otherwise (pageable arrays) the batch is cut into chunks; chunk k is copied in,
// evaluated and copied out on stream k % 2, so that the copies of one chunk overlap the kernel of the next.
// Device buffers and streams are kept per device; calls on the same device are serialised by a mutex.
#include <climits>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/matfun_cuda.h"
#include "mf_launch.h"

namespace {

constexpr int MAX_DEV = 64;

struct DevState {
  std::mutex mu;
  bool ready = false;
  cudaStream_t st[2] = {nullptr, nullptr};
  double *buf = nullptr;     // two chunk slots: input, F, J, H each
  size_t buf_doubles = 0;
  int *asym = nullptr;       // count of non-symmetric matrices (smf_eval_matrix)
};
DevState g_dev[MAX_DEV];

enum Fam { VOIGT = 0, MATRIX = 1, GENERAL = 2 };

int64_t chunk_for(int order) { return order == 2 ? (int64_t)1 << 16 : (order == 1 ? (int64_t)1 << 18 : (int64_t)1 << 20); }

cudaError_t ensure(DevState &d, size_t doubles) {
  if (!d.ready) {
    for (int s = 0; s < 2; s++) {
      const cudaError_t e = cudaStreamCreateWithFlags(&d.st[s], cudaStreamNonBlocking);
      if (e != cudaSuccess) return e;
    }
    const cudaError_t e = cudaMalloc(&d.asym, sizeof(int));
    if (e != cudaSuccess) return e;
    d.ready = true;
  }
  if (d.buf_doubles < doubles) {
    if (d.buf) cudaFree(d.buf);
    d.buf = nullptr;
    d.buf_doubles = 0;
    const cudaError_t e = cudaMalloc(&d.buf, doubles * sizeof(double));
    if (e != cudaSuccess) return e;
    d.buf_doubles = doubles;
  }
  return cudaSuccess;
}

cudaError_t launch(int fam, int kind, double alpha, int64_t n, const double *x, double *F, double *J, double *H,
                   cudaStream_t st, int *asym, bool reorder = true) {
  if (fam == GENERAL) {
    switch (kind) {
      case SMF_EXP: return mf::gmf_launch_exp(alpha, n, x, F, J, H, st, reorder);
      case SMF_LOG: return mf::gmf_launch_log(alpha, n, x, F, J, H, st, reorder);
      default: return mf::gmf_launch_pow(alpha, n, x, F, J, H, st, reorder);
    }
  }
  const bool mat = fam == MATRIX;
  switch (kind) {
    case SMF_EXP: return mf::smf_launch_exp(alpha, n, x, mat, F, J, H, st, asym, reorder);
    case SMF_LOG: return mf::smf_launch_log(alpha, n, x, mat, F, J, H, st, asym, reorder);
    case SMF_SQRT: return mf::smf_launch_sqrt(alpha, n, x, mat, F, J, H, st, asym, reorder);
    default: return mf::smf_launch_pow(alpha, n, x, mat, F, J, H, st, asym, reorder);
  }
}

// the device address of a page-locked, mapped host array (null for a null pointer); false for anything else
bool mapped(const void *p, void **dev) {
  *dev = nullptr;
  if (!p) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
  *dev = a.devicePointer;
  return true;
}

int host_eval(int fam, int kind, double alpha, int64_t n, const double *x, double *F, double *J, double *H) {
  // argument checks and normalisation of c/src/matfun.cc:23-32
  if (kind < SMF_EXP || kind > SMF_SQRT || n < 0 || (H && !J) || (kind == SMF_POW && !(alpha > 0))) return -1;
  if (n > 0 && (!x || !F)) return -1;
  if (fam == GENERAL && kind == SMF_SQRT) kind = SMF_POW, alpha = 0.5;
  if (kind != SMF_POW) alpha = kind == SMF_SQRT ? 0.5 : 0.0;
  if (n == 0) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return -2;
  DevState &d = g_dev[dev];
  std::lock_guard<std::mutex> lock(d.mu);
  const int order = H ? 2 : (J ? 1 : 0);
  const int64_t nin = fam == VOIGT ? 6 : 9, nf = nin, nj = J ? nf * nf : 0, nh = H ? nf * nf * nf : 0;
  void *mx, *mF, *mJ, *mH;
  if (mapped(x, &mx) & mapped(F, &mF) & mapped(J, &mJ) & mapped(H, &mH)) {
    // in place over the host link: launches of at most 2^26 matrices on one stream, then one synchronisation
    if (ensure(d, 0) != cudaSuccess) return -2;
    cudaStream_t st = d.st[0];
    cudaError_t e = fam == MATRIX ? cudaMemsetAsync(d.asym, 0, sizeof(int), st) : cudaSuccess;
    const int64_t step = (int64_t)1 << 26;
    for (int64_t lo = 0; lo < n && e == cudaSuccess; lo += step) {
      const int64_t m = n - lo < step ? n - lo : step;
      // (no batch-wide reordering here: its scratch would cross the host link twice)
      e = launch(fam, kind, alpha, m, (const double *)mx + lo * nin, (double *)mF + lo * nf,
                 J ? (double *)mJ + lo * nj : nullptr, H ? (double *)mH + lo * nh : nullptr, st,
                 fam == MATRIX ? d.asym : nullptr, false);
    }
    int asym = 0;
    if (e == cudaSuccess && fam == MATRIX) e = cudaMemcpyAsync(&asym, d.asym, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e != cudaSuccess || es != cudaSuccess) return -2;
    return asym ? -3 : 0;
  }
  const int64_t C = n < chunk_for(order) ? n : chunk_for(order);
  const int64_t per = nin + nf + nj + nh;
  if (ensure(d, (size_t)(2 * C * per)) != cudaSuccess) return -2;
  cudaError_t e = cudaSuccess;
  if (fam == MATRIX) e = cudaMemsetAsync(d.asym, 0, sizeof(int), d.st[0]);
  cudaEvent_t zeroed;
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&zeroed, cudaEventDisableTiming);
  if (e != cudaSuccess) return -2;
  cudaEventRecord(zeroed, d.st[0]);
  cudaStreamWaitEvent(d.st[1], zeroed, 0);
  for (int64_t lo = 0, k = 0; lo < n && e == cudaSuccess; lo += C, k++) {
    const int s = (int)(k & 1);
    const int64_t m = n - lo < C ? n - lo : C;
    double *dx = d.buf + (size_t)s * C * per, *dF = dx + C * nin, *dJ = dF + C * nf, *dH = dJ + C * nj;
    cudaStream_t st = d.st[s];
    e = cudaMemcpyAsync(dx, x + lo * nin, m * nin * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = launch(fam, kind, alpha, m, dx, dF, J ? dJ : nullptr, H ? dH : nullptr, st, fam == MATRIX ? d.asym : nullptr);
    if (e == cudaSuccess) e = cudaMemcpyAsync(F + lo * nf, dF, m * nf * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && J) e = cudaMemcpyAsync(J + lo * nj, dJ, m * nj * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && H) e = cudaMemcpyAsync(H + lo * nh, dH, m * nh * sizeof(double), cudaMemcpyDeviceToHost, st);
  }
  int asym = 0;
  if (e == cudaSuccess && fam == MATRIX) {
    cudaEvent_t done1;
    e = cudaEventCreateWithFlags(&done1, cudaEventDisableTiming);
    if (e == cudaSuccess) {
      cudaEventRecord(done1, d.st[1]);
      cudaStreamWaitEvent(d.st[0], done1, 0);
      e = cudaMemcpyAsync(&asym, d.asym, sizeof(int), cudaMemcpyDeviceToHost, d.st[0]);
      cudaEventDestroy(done1);
    }
  }
  const cudaError_t e0 = cudaStreamSynchronize(d.st[0]), e1 = cudaStreamSynchronize(d.st[1]);
  cudaEventDestroy(zeroed);
  if (e != cudaSuccess || e0 != cudaSuccess || e1 != cudaSuccess) return -2;
  return asym ? -3 : 0;
}

}  // namespace

extern "C" int smf_cuda_eval_host(int kind, double alpha, int64_t n, const double *v, double *F, double *J,
                                  double *H) {
  return host_eval(VOIGT, kind, alpha, n, v, F, J, H);
}

extern "C" int smf_cuda_eval_matrix_host(int kind, double alpha, int64_t n, const double *A, double *F, double *J,
                                         double *H) {
  return host_eval(MATRIX, kind, alpha, n, A, F, J, H);
}

extern "C" int gmf_cuda_eval_host(int kind, double alpha, int64_t n, const double *A, double *F, double *J,
                                  double *H) {
  return host_eval(GENERAL, kind, alpha, n, A, F, J, H);
}

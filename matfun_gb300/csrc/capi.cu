// capi.cu -- the C ABI of include/matfun_cuda.h: argument checks, normalisation of kind / alpha, grid limits and
// return codes as the reference's launchers (cuda/src/matfun_cuda.cu:119-141 launch, :169-190 glaunch), then the
// launch of the per-kind kernels (smf_<kind>.cu, gmf_<kind>.cu).
#include <atomic>
#include <climits>
#include <cstdint>

#include "../../include/matfun_cuda.h"
#include "mf_launch.h"

namespace {

constexpr int64_t SMF_MAX_N = (int64_t)INT_MAX * 32;  // the reference's grid limit: 2^31 - 1 blocks of 32
constexpr int64_t GMF_MAX_N = (int64_t)INT_MAX * 64;  // 2^31 - 1 blocks of 64

bool bad_args(int kind, double alpha, int64_t n, const double *x, const double *F, const double *J, const double *H) {
  if (kind < SMF_EXP || kind > SMF_SQRT || n < 0 || (H && !J) || (kind == SMF_POW && !(alpha > 0))) return true;
  return n > 0 && (!x || !F);
}

int smf_call(int kind, double alpha, int64_t n, const double *x, bool mat, double *F, double *J, double *H,
             cudaStream_t st, cudaError_t *err) {
  if (bad_args(kind, alpha, n, x, F, J, H)) return -1;
  if (kind != SMF_POW) alpha = kind == SMF_SQRT ? 0.5 : 0.0;
  if (n == 0) return 0;
  if (n > SMF_MAX_N) return -2;
  cudaError_t e;
  switch (kind) {
    case SMF_EXP: e = mf::smf_launch_exp(alpha, n, x, mat, F, J, H, st); break;
    case SMF_LOG: e = mf::smf_launch_log(alpha, n, x, mat, F, J, H, st); break;
    case SMF_SQRT: e = mf::smf_launch_sqrt(alpha, n, x, mat, F, J, H, st); break;
    default: e = mf::smf_launch_pow(alpha, n, x, mat, F, J, H, st); break;
  }
  if (err) *err = e;
  return e == cudaSuccess ? 0 : -2;
}

int gmf_call(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H, cudaStream_t st,
             cudaError_t *err) {
  if (bad_args(kind, alpha, n, A, F, J, H)) return -1;
  if (kind == SMF_SQRT) kind = SMF_POW, alpha = 0.5;
  if (kind != SMF_POW) alpha = 0.0;
  if (n == 0) return 0;
  if (n > GMF_MAX_N) return -2;
  cudaError_t e;
  switch (kind) {
    case SMF_EXP: e = mf::gmf_launch_exp(alpha, n, A, F, J, H, st); break;
    case SMF_LOG: e = mf::gmf_launch_log(alpha, n, A, F, J, H, st); break;
    default: e = mf::gmf_launch_pow(alpha, n, A, F, J, H, st); break;
  }
  if (err) *err = e;
  return e == cudaSuccess ? 0 : -2;
}

}  // namespace

int mf::eval_f64(int family, int kind, double alpha, int64_t n, const double *x, double *F, double *J, double *H,
                 cudaStream_t st, cudaError_t *err) {
  if (err) *err = cudaSuccess;
  return family == 2 ? gmf_call(kind, alpha, n, x, F, J, H, st, err)
                     : smf_call(kind, alpha, n, x, family == 1, F, J, H, st, err);
}

extern "C" int smf_cuda_eval(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H,
                             void *stream) {
  return mf::eval_f64(0, kind, alpha, n, v, F, J, H, (cudaStream_t)stream, nullptr);
}

extern "C" int smf_cuda_eval_matrix(int kind, double alpha, int64_t n, const double *A, double *F, double *J,
                                    double *H, void *stream) {
  return mf::eval_f64(1, kind, alpha, n, A, F, J, H, (cudaStream_t)stream, nullptr);
}

extern "C" int gmf_cuda_eval(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H,
                             void *stream) {
  return mf::eval_f64(2, kind, alpha, n, A, F, J, H, (cudaStream_t)stream, nullptr);
}

extern "C" int gmf_cuda_tangent(int kind, double alpha, int64_t n, const double *A, double *F, double *G, double *K,
                                void *stream) {
  if (kind < SMF_EXP || kind > SMF_SQRT || n < 0 || (kind == SMF_POW && !(alpha > 0))) return -1;
  if (n > 0 && (!A || !K)) return -1;
  if (kind == SMF_SQRT) kind = SMF_POW, alpha = 0.5;
  if (kind != SMF_POW) alpha = 0.0;
  if (n == 0) return 0;
  if (n > GMF_MAX_N) return -2;
  const cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  switch (kind) {
    case SMF_EXP: e = mf::gmf_tangent_launch_exp(alpha, n, A, F, G, K, st); break;
    case SMF_LOG: e = mf::gmf_tangent_launch_log(alpha, n, A, F, G, K, st); break;
    default: e = mf::gmf_tangent_launch_pow(alpha, n, A, F, G, K, st); break;
  }
  return e == cudaSuccess ? 0 : -2;
}

namespace {
int smf_call_f32(int kind, double alpha, int64_t n, const float *x, bool mat, float *F, float *J, float *H,
                 void *stream) {
  if (kind < SMF_EXP || kind > SMF_SQRT || n < 0 || (H && !J) || (kind == SMF_POW && !(alpha > 0))) return -1;
  if (n > 0 && (!x || !F)) return -1;
  if (kind != SMF_POW) alpha = kind == SMF_SQRT ? 0.5 : 0.0;
  if (n == 0) return 0;
  if (n > SMF_MAX_N) return -2;
  const cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  switch (kind) {
    case SMF_EXP: e = mf::smf_mixed_launch_exp(alpha, n, x, mat, F, J, H, st); break;
    case SMF_LOG: e = mf::smf_mixed_launch_log(alpha, n, x, mat, F, J, H, st); break;
    case SMF_SQRT: e = mf::smf_mixed_launch_sqrt(alpha, n, x, mat, F, J, H, st); break;
    default: e = mf::smf_mixed_launch_pow(alpha, n, x, mat, F, J, H, st); break;
  }
  return e == cudaSuccess ? 0 : -2;
}
}  // namespace

extern "C" int smf_cuda_eval_f32(int kind, double alpha, int64_t n, const float *v, float *F, float *J, float *H,
                                 void *stream) {
  return smf_call_f32(kind, alpha, n, v, false, F, J, H, stream);
}

namespace mf {
std::atomic<int> smf_voigt_variant[2] = {{2}, {1}};  // the store path of the FP32 Voigt kernels at orders 1, 2
}

extern "C" int matfun_cuda_smf_f32_tune(int order, int variant) {
  if (order < 1 || order > 2 || variant < 0 || variant > 3) return -1;
  mf::smf_voigt_variant[order - 1] = variant;
  return 0;
}

extern "C" int smf_cuda_eval_matrix_f32(int kind, double alpha, int64_t n, const float *A, float *F, float *J,
                                        float *H, void *stream) {
  return smf_call_f32(kind, alpha, n, A, true, F, J, H, stream);
}

extern "C" int gmf_cuda_eval_f32(int kind, double alpha, int64_t n, const float *A, float *F, float *J, float *H,
                                 void *stream) {
  if (kind < SMF_EXP || kind > SMF_SQRT || n < 0 || (H && !J) || (kind == SMF_POW && !(alpha > 0))) return -1;
  if (n > 0 && (!A || !F)) return -1;
  if (kind == SMF_SQRT) kind = SMF_POW, alpha = 0.5;
  if (kind != SMF_POW) alpha = 0.0;
  if (n == 0) return 0;
  if (n > GMF_MAX_N) return -2;
  const cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  switch (kind) {
    case SMF_EXP: e = mf::gmf_mixed_launch_exp(alpha, n, A, F, J, H, st); break;
    case SMF_LOG: e = mf::gmf_mixed_launch_log(alpha, n, A, F, J, H, st); break;
    default: e = mf::gmf_mixed_launch_pow(alpha, n, A, F, J, H, st); break;
  }
  return e == cudaSuccess ? 0 : -2;
}

namespace {
cudaError_t adjoint_launch(bool general, int kind, double al, int64_t n, const double *A, const double *W,
                           const double *V, double *F, double *Abar, double *JV, double *HWV, cudaStream_t st) {
  return general ? mf::gmf_adjoint_launch(kind, al, n, A, W, V, F, Abar, JV, HWV, st)
                 : mf::smf_adjoint_launch(kind, al, n, A, W, V, F, Abar, JV, HWV, st);
}
cudaError_t adjoint_launch(bool general, int kind, double al, int64_t n, const float *A, const float *W,
                           const float *V, float *F, float *Abar, float *JV, float *HWV, cudaStream_t st) {
  return general ? mf::gmf_adjoint_launch_f32(kind, al, n, A, W, V, F, Abar, JV, HWV, st)
                 : mf::smf_adjoint_launch_f32(kind, al, n, A, W, V, F, Abar, JV, HWV, st);
}

template <typename T>
int adjoint_call(bool general, int kind, double alpha, int64_t n, const T *A, const T *W, const T *V, T *F, T *Abar,
                 T *JV, T *HWV, void *stream) {
  if (kind < SMF_EXP || kind > SMF_SQRT || n < 0 || (kind == SMF_POW && !(alpha > 0))) return -1;
  if ((Abar && !W) || (JV && !V) || (HWV && !(W && V))) return -1;
  if (n > 0 && !A) return -1;
  if (general && kind == SMF_SQRT) kind = SMF_POW, alpha = 0.5;
  if (kind != SMF_POW) alpha = kind == SMF_SQRT ? 0.5 : 0.0;
  if (n == 0 || !(F || Abar || JV || HWV)) return 0;
  if (n > SMF_MAX_N) return -2;
  const cudaError_t e = adjoint_launch(general, kind, alpha, n, A, W, V, F, Abar, JV, HWV, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : -2;
}
}  // namespace

extern "C" int gmf_cuda_adjoint(int kind, double alpha, int64_t n, const double *A, const double *W, const double *V,
                                double *F, double *Abar, double *JV, double *HWV, void *stream) {
  return adjoint_call(true, kind, alpha, n, A, W, V, F, Abar, JV, HWV, stream);
}

extern "C" int smf_cuda_adjoint(int kind, double alpha, int64_t n, const double *A, const double *W, const double *V,
                                double *F, double *Abar, double *JV, double *HWV, void *stream) {
  return adjoint_call(false, kind, alpha, n, A, W, V, F, Abar, JV, HWV, stream);
}

extern "C" const char *matfun_cuda_version(void) { return "matfun-gb300 0.1.0 (sm_103a)"; }

extern "C" int gmf_cuda_adjoint_f32(int kind, double alpha, int64_t n, const float *A, const float *W, const float *V,
                                    float *F, float *Abar, float *JV, float *HWV, void *stream) {
  return adjoint_call(true, kind, alpha, n, A, W, V, F, Abar, JV, HWV, stream);
}

extern "C" int smf_cuda_adjoint_f32(int kind, double alpha, int64_t n, const float *A, const float *W, const float *V,
                                    float *F, float *Abar, float *JV, float *HWV, void *stream) {
  return adjoint_call(false, kind, alpha, n, A, W, V, F, Abar, JV, HWV, stream);
}

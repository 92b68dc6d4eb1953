/* matfun_shim.c -- libmatfun.so of this package: the reference's CPU C API (c/include/matfun/matfun.h:28-53 --
 * smf_eval, smf_eval_matrix, gmf_eval, smf_simd_name, smf_version) with the GPU behind it, so that the reference's
 * own front ends (python/src/matfun/_capi.py via MATFUN_LIB, C callers linking -lmatfun) run on the GB300 unchanged.
 * Each call forwards to the host-buffer entry points of libmatfun_cuda.so (include/matfun_cuda.h). */
#include <stdint.h>

int smf_cuda_eval_host(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H);
int smf_cuda_eval_matrix_host(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H);
int gmf_cuda_eval_host(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H);

int smf_eval(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H) {
  return smf_cuda_eval_host(kind, alpha, n, v, F, J, H);
}
int smf_eval_matrix(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H) {
  return smf_cuda_eval_matrix_host(kind, alpha, n, A, F, J, H);
}
int gmf_eval(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H) {
  return gmf_cuda_eval_host(kind, alpha, n, A, F, J, H);
}
const char *smf_simd_name(void) { return "cuda-sm_103a"; }
const char *smf_version(void) { return "0.1.3"; }

/* matfun.h -- the reference's CPU C API (c/include/matfun/matfun.h:28-53 of BodeTobias/matfun), exported by this
 * package's libmatfun.so (matfun_gb300/shim/matfun_shim.c) with the GPU behind it: host arrays, synchronous,
 * return codes 0 / -1 (invalid arguments) / -3 (smf_eval_matrix: a matrix not symmetric, its results NaN), and -2 for
 * a CUDA error.  Layouts as in include/matfun_cuda.h. */
#ifndef MATFUN_GB300_HOST_H
#define MATFUN_GB300_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* replaces smf_eval (c/include/matfun/matfun.h:33) */
int smf_eval(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H);
/* replaces smf_eval_matrix (c/include/matfun/matfun.h:37) */
int smf_eval_matrix(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H);
/* replaces gmf_eval (c/include/matfun/matfun.h:47) */
int gmf_eval(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H);
/* replaces smf_simd_name (c/include/matfun/matfun.h:51): "cuda-sm_103a" */
const char *smf_simd_name(void);
/* replaces smf_version (c/include/matfun/matfun.h:53) */
const char *smf_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MATFUN_GB300_HOST_H */

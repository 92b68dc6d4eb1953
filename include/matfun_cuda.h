/* matfun_cuda.h -- C ABI of libmatfun_cuda (GB300 / sm_103a build): batched 3x3 matrix functions exp, log, sqrt and
 * A^alpha with first and second derivatives, on the GPU.
 *
 * Drop-in for the reference's CUDA library: the same three entry points, argument meaning, layouts and return codes
 * as cuda/include/matfun/matfun_cuda.h:16-22 of BodeTobias/matfun (layouts: c/include/matfun/matfun.h:1-41).
 *
 * Conventions (unchanged from the reference):
 *   - all arrays are DEVICE pointers owned by the caller, row-major, one matrix after the other;
 *   - the work is queued on `stream` (a cudaStream_t, NULL = default stream) and the call returns without waiting;
 *   - J and H may be NULL (H needs J); F is required;
 *   - returns 0; -1 for invalid arguments (unknown kind, n < 0, H without J, alpha <= 0 for SMF_POW, and in this
 *     build also a NULL input or F pointer with n > 0); -2 for a CUDA launch error or a grid the reference could not
 *     launch (n > 32 (2^31 - 1) for smf, n > 64 (2^31 - 1) for gmf) -- then nothing is launched and no CUDA error
 *     stays pending;
 *   - n == 0 returns 0 without a launch;
 *   - a matrix outside the domain (gmf: a real eigenvalue <= 0 for log / sqrt / pow) or a non-symmetric matrix in
 *     smf_cuda_eval_matrix (|A_ij - A_ji| > 1e-8 max|A_kl|) gives NaN results for that matrix only.
 *
 * Layouts:
 *   smf_cuda_eval         v (n, 6) Voigt (A11, A22, A33, A12, A13, A23) -> F (n, 6), J (n, 6, 6), H (n, 6, 6, 6)
 *   smf_cuda_eval_matrix  A (n, 3, 3) symmetric -> F (n, 3, 3), J (n, 3,3,3,3), H (n, 3,3,3,3,3,3), the derivatives of
 *                         A -> f((A + A^T) / 2)
 *   gmf_cuda_eval         A (n, 3, 3) general -> F, J, H as above, the full derivatives, principal branch
 */
#ifndef MATFUN_GB300_CUDA_H
#define MATFUN_GB300_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* kind codes: c/include/matfun/matfun.h:28 */
#ifndef MATFUN_H
enum smf_kind { SMF_EXP = 0, SMF_LOG = 1, SMF_POW = 2, SMF_SQRT = 3 };
#endif

/* replaces smf_cuda_eval, cuda/include/matfun/matfun_cuda.h:16 (implementation cuda/src/matfun_cuda.cu:199-202) */
int smf_cuda_eval(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H, void *stream);

/* replaces smf_cuda_eval_matrix, cuda/include/matfun/matfun_cuda.h:18-19 (cuda/src/matfun_cuda.cu:204-207) */
int smf_cuda_eval_matrix(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H,
                         void *stream);

/* replaces gmf_cuda_eval, cuda/include/matfun/matfun_cuda.h:22 (cuda/src/matfun_cuda.cu:194-197) */
int gmf_cuda_eval(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H, void *stream);

/* Mixed precision (no counterpart in the reference): FP32 arrays in and out, the bulk of the arithmetic in FP32.
 * smf: no FP64 arithmetic at all; the deviator, the Rayleigh quotients that give the eigenvalues and the eigenvalue
 * differences of the near-coalescent divided-difference branches run in float-float (two FP32 words, about 48
 * significant bits) on the FP32 pipe.  gmf: the spectral analysis (closed-form roots, refinement, branch-cut pair,
 * groups) and the residues run in FP64, the confluent series in float-float; storage and the J / H assembly in FP32.
 * Same layouts, kinds and return codes as smf_cuda_eval / smf_cuda_eval_matrix / gmf_cuda_eval.  Error against the
 * FP64 results of the same FP32 input values, per matrix (max |x - ref| / max |ref| over each matrix's F, J or H),
 * on the tested workloads: <= 1e-6 for every kind and order wherever the outputs fit FP32's range. */
int smf_cuda_eval_f32(int kind, double alpha, int64_t n, const float *v, float *F, float *J, float *H, void *stream);
int smf_cuda_eval_matrix_f32(int kind, double alpha, int64_t n, const float *A, float *F, float *J, float *H,
                             void *stream);
int gmf_cuda_eval_f32(int kind, double alpha, int64_t n, const float *A, float *F, float *J, float *H, void *stream);
/* Store path of smf_cuda_eval_f32 at order 1 or 2 (no counterpart in the reference; chosen by the autotuner,
 * matfun_gb300/autotune.py): 0 = per-entry stores of the expanded rows; 1 = J / H rows staged in shared-memory boxes
 * of 32 rows x 128 bytes and written by the TMA unit; 2 = the same with boxes of 32 rows x 64 bytes (less shared
 * memory and fewer registers per thread, more resident warps); 3 = 64-byte boxes with fewer registers per thread and
 * more resident warps than 2 at order 2.  Defaults: 2 at order 1, 1 at order 2.  J and H must be 16-byte aligned for
 * 1-3, else the call takes path 0.  Results agree to FP32 rounding.  Returns 0 or -1 (unknown order or path). */
int matfun_cuda_smf_f32_tune(int order, int variant);

/* Adjoints (no counterpart in the reference): contractions of J and H with directions, without
 * forming J or H.  Matrix layout (n, 3, 3) for every array; W, V device arrays of directions; outputs, each optional:
 *   F    = f(A)
 *   Abar = J^T W    (Abar_cd = sum_ab W_ab dF_ab/dA_cd: the gradient of sum <W, f(A)>)     needs W
 *   JV   = J V      ((JV)_ab = sum_cd dF_ab/dA_cd V_cd: the derivative of f(A) along V)    needs V
 *   HWV  = W.H.V    (HWV_ef = sum_abcd W_ab d2F_ab/dA_cd dA_ef V_cd)                       needs W and V
 * smf_cuda_adjoint treats A as symmetric (the derivatives of A -> f((A + A^T)/2), as smf_cuda_eval_matrix).
 * Returns 0, -1 (invalid kind / alpha, n < 0, an output without its directions), -2 (CUDA error). */
int smf_cuda_adjoint(int kind, double alpha, int64_t n, const double *A, const double *W, const double *V, double *F,
                     double *Abar, double *JV, double *HWV, void *stream);
int gmf_cuda_adjoint(int kind, double alpha, int64_t n, const double *A, const double *W, const double *V, double *F,
                     double *Abar, double *JV, double *HWV, void *stream);
/* The adjoints in mixed precision: FP32 arrays; gmf from its FP64 record rounded once, smf from the eigensystem and
 * divided differences of smf_cuda_eval_f32; contractions in FP32.  Same arguments and return codes. */
int smf_cuda_adjoint_f32(int kind, double alpha, int64_t n, const float *A, const float *W, const float *V, float *F,
                         float *Abar, float *JV, float *HWV, void *stream);
int gmf_cuda_adjoint_f32(int kind, double alpha, int64_t n, const float *A, const float *W, const float *V, float *F,
                         float *Abar, float *JV, float *HWV, void *stream);

/* Tangent of psi(A) = |f(A)|^2 / 2 (no counterpart in the reference; the consumer-side contraction of the
 * reference's theory.md:190, e.g. the Hencky-type potential |log A|^2 / 2 of a Newton method), general family, FP64,
 * matrix layout, without forming J or H:
 *   F = f(A)                      (n, 3, 3), optional
 *   G = J^T F                     (n, 3, 3), optional: G_cd = sum_ab F_ab dF_ab/dA_cd, the gradient of psi
 *   K = J^T J + F : H             (n, 9, 9): K_{cd,ef} = sum_ab (dF_ab/dA_cd dF_ab/dA_ef + F_ab d2F_ab/dA_cd dA_ef),
 *                                 the Hessian of psi (symmetric)
 * Returns 0, -1 (invalid kind / alpha, n < 0, A or K missing for n > 0), -2 (CUDA error).  Asynchronous on
 * `stream`; allocates nothing (the batch order's scratch lies in K's last rows, evaluated afterwards). */
int gmf_cuda_tangent(int kind, double alpha, int64_t n, const double *A, double *F, double *G, double *K, void *stream);

/* Batched evaluation (no counterpart in the reference): many requests of uneven size and
 * mixed family / kind / order / precision in ONE launch of a persistent kernel.  A request: */
typedef struct mf_request {
  int32_t family;  /* 0: smf Voigt (smf_cuda_eval), 1: smf matrix (smf_cuda_eval_matrix), 2: gmf (gmf_cuda_eval) */
  int32_t kind;    /* SMF_EXP, SMF_LOG, SMF_POW, SMF_SQRT */
  int32_t order;   /* 0: F; 1: F, J; 2: F, J, H */
  int32_t dtype;   /* 0: FP64 arrays; 1: FP32 arrays (the mixed-precision paths) */
  double alpha;    /* exponent of SMF_POW */
  int64_t n;       /* matrices */
  const void *x;   /* device input, layouts as above */
  void *F, *J, *H; /* device outputs (J for order >= 1, H for order 2) */
} mf_request;

/* All requests queued on `stream` as one launch of the persistent kernel (the request table is uploaded on `stream`
 * first; gmf requests of log / pow at orders 1-2 with >= 2048 matrices are first ordered by spectral class, three
 * small kernels each, as the single gmf entry point orders large batches).  Returns 0, -1 when a request breaks the
 * rules of its single entry point or `stream` is being captured into a CUDA graph (then nothing runs: the table is
 * uploaded from a host copy that lives only during the call; capture matfun_cuda_batched_run instead), -2 for a CUDA
 * error.  Results equal those of the single entry points to rounding (1e-13 relative, FP64). */
int matfun_cuda_batched(const mf_request *requests, int count, void *stream);
/* The same as a plan: the table is validated and uploaded once (synchronously); matfun_cuda_batched_run then only
 * clears the tile cursor and launches, so it can be captured in a CUDA graph and replayed.  The arrays the requests
 * name must stay allocated while the plan is used. */
int matfun_cuda_batched_plan(const mf_request *requests, int count, void **plan);
int matfun_cuda_batched_run(void *plan, void *stream);
int matfun_cuda_batched_free(void *plan);
/* No counterpart in the reference.  matfun_cuda_batched without any device allocation, for callers that cannot call
 * cudaMalloc (a framework that owns all device memory through its own allocator, a plugin that is only handed device
 * arrays): the request table and the tile cursor go into one fixed 256 KiB array of device memory that belongs to the
 * library image (present on every GPU that uses the library, until the process exits) instead of a buffer allocated
 * on first use.  The first call on a device looks up that array's device address (cudaGetSymbolAddress) with the
 * device current; make that first call before capturing a stream.  All calls share the array and it keeps the last
 * call's table: calls whose launches overlap on the GPU (different streams, no ordering between them) race and give
 * wrong results.  Calls from several host threads on one stream are queued whole, one after the other (a lock covers
 * the table copy and the launch).  Returns 0, -1 (an invalid request, or `stream` is being captured: the table is
 * copied from a host copy that lives only during the call), -2 (CUDA error), -4 (the table -- 72 bytes per request
 * plus its coefficients, about 2.5 KB for gmf and 0.3 KB for smf -- does not fit the 256 KiB). */
int matfun_cuda_batched_noalloc(const mf_request *requests, int count, void *stream);

/* Tuning of the persistent launch (set by the autotuner, matfun_gb300/autotune.py): CTAs per SM (1..8) and whether
 * requests are laid out longest first (1) or as given (0).  Returns 0 or -1. */
int matfun_cuda_batched_tune(int ctas_per_sm, int longest_first);

/* Matrices per tile of the symmetric-family requests of later batched tables: 128 (default) or 64; the general family
 * always takes 128.  A 64-matrix tile needs half the shared memory of a 128-matrix one, its per-matrix phase runs on
 * half of the CTA's 128 threads.  Returns 0 or -1. */
int matfun_cuda_batched_tune_tiles(int smf_tile);

/* Host-buffer forms: the reference's CPU entry points smf_eval, smf_eval_matrix and gmf_eval
 * (c/include/matfun/matfun.h:28-41; implementation c/src/matfun.cc:87-97) evaluated on the current GPU: HOST arrays
 * in and out, synchronous, same return codes as the CPU library (0, -1 invalid arguments, -3 when a matrix given to
 * smf_cuda_eval_matrix_host is not symmetric -- its results are NaN), and -2 for a CUDA error.  The batch is
 * streamed through the GPU in chunks on two streams, so copies overlap the kernels; page-locked host arrays make the
 * copies fastest.  libmatfun.so of this package exports the same functions under the reference's names. */
int smf_cuda_eval_host(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H);
int smf_cuda_eval_matrix_host(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H);
int gmf_cuda_eval_host(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H);

/* XLA FFI custom-call handlers registered by matfun.jax for the CUDA platform (reference:
 * cuda/src/matfun_cuda.cu:245-261, bound by name in python/src/matfun/jax.py:66-87 as targets matfun_value,
 * matfun_value_jac, matfun_value_jac_hess, matfun_matrix_value*, matfun_gen_value*).  Argument: XLA's call frame
 * (XLA FFI C API 0.1); result: NULL on success, else an XLA error created through the frame's API.  On XLA's stream:
 * input x (F64, (..., 6) Voigt or (..., 3, 3)), results F, (F, J) or (F, J, H) as F64 buffers, attributes kind
 * (int64) and alpha (double). */
void *SmfValueCuda(void *call_frame);
void *SmfValueJacCuda(void *call_frame);
void *SmfValueJacHessCuda(void *call_frame);
void *SmfMatrixValueCuda(void *call_frame);
void *SmfMatrixValueJacCuda(void *call_frame);
void *SmfMatrixValueJacHessCuda(void *call_frame);
void *GmfValueCuda(void *call_frame);
void *GmfValueJacCuda(void *call_frame);
void *GmfValueJacHessCuda(void *call_frame);

/* Additional XLA FFI handlers (no counterpart in the reference), same call-frame conventions:
 *   SmfValueF32Cuda, SmfMatrixValueF32Cuda, GmfValueF32Cuda: the FP32 forms (smf_cuda_eval_f32 ...), F32 buffers,
 *     one to three results (F, J, H), attributes kind, alpha;
 *   SmfAdjointCuda, GmfAdjointCuda (F64) and SmfAdjointF32Cuda, GmfAdjointF32Cuda (F32): arguments A, W, V
 *     ((..., 3, 3); W or V with no elements when not given), attributes kind, alpha and outputs (int64 bit mask:
 *     1 F, 2 J^T W, 4 J V, 8 W.H.V), one result per set bit in that order (smf_cuda_adjoint / gmf_cuda_adjoint);
 *   GmfTangentCuda (F64): argument A, attributes kind, alpha and outputs (1 F, 2 G = J^T F, 4 K = J^T J + F : H;
 *     K required), one result per set bit in that order, F and G of A's shape, K with 9 times its elements
 *     (gmf_cuda_tangent). */
void *SmfValueF32Cuda(void *call_frame);
void *SmfMatrixValueF32Cuda(void *call_frame);
void *GmfValueF32Cuda(void *call_frame);
void *SmfAdjointCuda(void *call_frame);
void *GmfAdjointCuda(void *call_frame);
void *SmfAdjointF32Cuda(void *call_frame);
void *GmfAdjointF32Cuda(void *call_frame);
void *GmfTangentCuda(void *call_frame);

/* XLA FFI API version the handlers implement, major * 1000 + minor (reference: cuda/src/matfun_cuda.cu:265) */
int smf_xla_ffi_api_version(void);

/* Diagnostics (no counterpart in the reference): the measured FP64 / FP32 fused-multiply-add throughput of the
 * current GPU in TFLOP/s (independent FMA chains on every SM), the pipe bounds of this library's kernels.
 * Synchronous.  Return 0, or -1 / -2 like the entry points above. */
int matfun_cuda_fp64_peak(double *tflops);
int matfun_cuda_fp32_peak(double *tflops);

/* version string of this library (no counterpart in the reference's CUDA header; cf. smf_version, matfun.h:51) */
const char *matfun_cuda_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MATFUN_GB300_CUDA_H */

// xla_ffi.cu -- the XLA FFI custom-call handlers that matfun.jax registers for the CUDA platform
// (cuda/src/matfun_cuda.cu:209-265; python/src/matfun/jax.py:66-87 binds them by name and checks
// smf_xla_ffi_api_version): SmfValueCuda ... GmfValueJacHessCuda; and, as additions, their FP32 forms
// (SmfValueF32Cuda, SmfMatrixValueF32Cuda, GmfValueF32Cuda: any number of results 1..3 as the F64 ones) and the
// adjoints (SmfAdjointCuda, GmfAdjointCuda and their F32 forms), which matfun_gb300.jax builds custom_vjp on.
//
// Each handler receives XLA's call frame for one custom call: on XLA's stream, the input buffer x (F64, Voigt (..., 6)
// or matrices (..., 3, 3)), one to three F64 result buffers F, J, H, and the scalar attributes kind (S64) and alpha
// (F64).  It checks the frame as the reference's binding does (structure size, metadata query, execution stage, the
// number of arguments and attributes, argument and attribute types, by name), then the shapes and the result count
// as its Eval (matfun_cuda.cu:220-243), and launches the same kernels as smf_cuda_eval / smf_cuda_eval_matrix /
// gmf_cuda_eval.  Errors go back as XLA errors: INVALID_ARGUMENT for a malformed call or an invalid kind / alpha,
// INTERNAL for a failed launch.  The frame is read through xla_ffi_abi.h; no XLA or JAX headers are needed.
#include <algorithm>
#include <cstring>
#include <string>

#include "../../include/matfun_cuda.h"
#include "mf_launch.h"
#include "xla_ffi_abi.h"

namespace {

enum { VOIGT = 0, MATRIX = 1, GENERAL = 2 };

void *make_error(const mfx_api *api, int errc, const std::string &msg) {
  mfx_error_create_args a;
  a.struct_size = MFX_ERROR_CREATE_ARGS_SIZE;
  a.extension_start = nullptr;
  a.message = msg.c_str();
  a.errc = errc;
  return api->error_create(&a);
}

void *invalid(const mfx_api *api, const std::string &msg) { return make_error(api, MFX_ERR_INVALID_ARGUMENT, msg); }

bool name_is(const mfx_bytespan *s, const char *name) {
  const size_t n = std::strlen(name);
  return s != nullptr && s->len == n && std::memcmp(s->ptr, name, n) == 0;
}

// the value of scalar attribute `name` of type dtype, or nullptr with the reason in why
const void *scalar_attr(const mfx_attrs &at, const char *name, int dtype, std::string &why) {
  for (int64_t i = 0; i < at.size; i++) {
    if (!name_is(at.names[i], name)) continue;
    const mfx_scalar *s = static_cast<const mfx_scalar *>(at.attrs[i]);
    if (at.types[i] != MFX_ATTR_SCALAR || s == nullptr || s->dtype != dtype) {
      why += std::string(why.empty() ? "" : "; ") + "wrong attribute type of `" + name + "`";
      return nullptr;
    }
    return s->value;
  }
  why += std::string(why.empty() ? "" : "; ") + "missing attribute `" + name + "`";
  return nullptr;
}

// a buffer of dtype dt (argument or result), or nullptr with the reason in why
const mfx_buffer *typed_buffer(int32_t type, void *p, int expected_type, int dt, const char *what, std::string &why) {
  const mfx_buffer *b = static_cast<const mfx_buffer *>(p);
  if (type != expected_type || b == nullptr) {
    why += std::string(why.empty() ? "" : "; ") + "wrong " + what + " type: expected a buffer";
    return nullptr;
  }
  if (b->dtype != dt) {
    why += std::string(why.empty() ? "" : "; ") + "wrong " + what + " dtype: expected " +
           (dt == MFX_DT_F64 ? "F64" : "F32") + " but got " + std::to_string(b->dtype);
    return nullptr;
  }
  return b;
}

int64_t elements(const mfx_buffer *b) {
  int64_t c = 1;
  for (int64_t d = 0; d < b->rank; d++) c *= b->dims[d];
  return c;
}

template <typename T>
constexpr int dtype_of() { return sizeof(T) == 8 ? MFX_DT_F64 : MFX_DT_F32; }

// the entry points by family and element type
int eval_t(int fam, int kind, double alpha, int64_t n, const double *x, double **p, cudaStream_t st, cudaError_t *err) {
  return mf::eval_f64(fam, kind, alpha, n, x, p[0], p[1], p[2], st, err);
}
int eval_t(int fam, int kind, double alpha, int64_t n, const float *x, float **p, cudaStream_t st, cudaError_t *err) {
  *err = cudaSuccess;
  return fam == 2 ? gmf_cuda_eval_f32(kind, alpha, n, x, p[0], p[1], p[2], st)
                  : (fam == 1 ? smf_cuda_eval_matrix_f32(kind, alpha, n, x, p[0], p[1], p[2], st)
                              : smf_cuda_eval_f32(kind, alpha, n, x, p[0], p[1], p[2], st));
}

void *metadata(const mfx_api *api, mfx_metadata_ext *ext) {
  if (ext->extension_base.struct_size < MFX_METADATA_EXT_SIZE || ext->metadata == nullptr ||
      ext->metadata->struct_size < MFX_METADATA_SIZE)
    return invalid(api, "Unexpected XLA_FFI_Metadata size. Check installed software versions.");
  ext->metadata->api_version.struct_size = MFX_API_VERSION_SIZE;
  ext->metadata->api_version.extension_start = nullptr;
  ext->metadata->api_version.major_version = MFX_API_MAJOR;
  ext->metadata->api_version.minor_version = MFX_API_MINOR;
  ext->metadata->traits = 0;
  return nullptr;
}

// the common checks of a call frame: size, metadata query, stage, argument and attribute counts; nullptr when the
// frame is to be decoded, else the result to return (*done set)
void *frame_checks(mfx_call_frame *cf, int64_t nargs, int64_t nattrs, bool *done) {
  const mfx_api *api = cf->api;
  *done = true;
  if (cf->struct_size != MFX_CALL_FRAME_SIZE)
    return invalid(api, "Unexpected XLA_FFI_CallFrame size: expected " + std::to_string(MFX_CALL_FRAME_SIZE) +
                            " got " + std::to_string(cf->struct_size) + ". Check installed software versions.");
  if (cf->extension_start != nullptr && cf->extension_start->type == MFX_EXT_METADATA)
    return metadata(api, reinterpret_cast<mfx_metadata_ext *>(cf->extension_start));
  if (cf->stage != MFX_STAGE_EXECUTE)
    return invalid(api, "Wrong execution stage: expected `3` but got `" + std::to_string(cf->stage) + "`");
  if (cf->args.size != nargs)
    return invalid(api, "Wrong number of arguments: expected " + std::to_string(nargs) + " but got " +
                            std::to_string(cf->args.size));
  if (cf->attrs.size != nattrs)
    return invalid(api, "Wrong number of attributes: expected " + std::to_string(nattrs) + " but got " +
                            std::to_string(cf->attrs.size));
  *done = false;
  return nullptr;
}

// XLA's stream of the call, or an error
void *get_stream(mfx_call_frame *cf, cudaStream_t *st) {
  mfx_stream_get_args sa;
  sa.struct_size = MFX_STREAM_GET_ARGS_SIZE;
  sa.extension_start = nullptr;
  sa.ctx = cf->ctx;
  sa.stream = nullptr;
  void *e = cf->api->stream_get(&sa);
  *st = (cudaStream_t)sa.stream;
  return e;
}

void *launch_error(const mfx_api *api, int res, cudaError_t err) {
  if (res == -1) return invalid(api, "matfun: invalid kind or alpha");
  if (res != 0)
    return make_error(api, MFX_ERR_INTERNAL, std::string("matfun: CUDA launch failed: ") +
                                                 (err == cudaSuccess ? "grid limit" : cudaGetErrorString(err)));
  return nullptr;
}

int clamp_kind(int64_t kind64) {  // out of the int range: invalid
  return (int)std::min<int64_t>(std::max<int64_t>(kind64, -1), SMF_SQRT + 1);
}

// x -> F, (F, J) or (F, J, H) of a family, as smf_cuda_eval / smf_cuda_eval_matrix / gmf_cuda_eval (T = double) or
// their FP32 forms (T = float)
template <int FAM, typename T>
void *handle(mfx_call_frame *cf) {
  const mfx_api *api = cf->api;
  bool done;
  if (void *r = frame_checks(cf, 1, 2, &done); done) return r;
  constexpr int DT = dtype_of<T>();
  // operands, in the order of the binding: XLA's stream, x, (the results), kind, alpha
  cudaStream_t st;
  if (void *e = get_stream(cf, &st)) return e;
  std::string why;
  const mfx_buffer *x = typed_buffer(cf->args.types[0], cf->args.args[0], MFX_ARG_BUFFER, DT, "argument", why);
  const void *kind_p = scalar_attr(cf->attrs, "kind", MFX_DT_S64, why);
  const void *alpha_p = scalar_attr(cf->attrs, "alpha", MFX_DT_F64, why);
  if (!why.empty()) return invalid(api, "Failed to decode all FFI handler operands: " + why);

  const int64_t r = x->rank;
  const bool shape_ok = FAM == VOIGT ? (r >= 1 && x->dims[r - 1] == 6)
                                     : (r >= 2 && x->dims[r - 1] == 3 && x->dims[r - 2] == 3);
  if (!shape_ok)
    return invalid(api, FAM == VOIGT ? "matfun: expected Voigt vectors of shape (..., 6)"
                                     : "matfun: expected matrices of shape (..., 3, 3)");
  if (cf->rets.size < 1 || cf->rets.size > 3) return invalid(api, "matfun: expected F, (F, J) or (F, J, H)");
  T *p[3] = {nullptr, nullptr, nullptr};
  for (int64_t i = 0; i < cf->rets.size; i++) {
    const mfx_buffer *b = typed_buffer(cf->rets.types[i], cf->rets.rets[i], MFX_RET_BUFFER, DT, "result", why);
    if (b == nullptr) return invalid(api, "Failed to decode result " + std::to_string(i) + ": " + why);
    p[i] = static_cast<T *>(b->data);
  }
  const int kind = clamp_kind(*static_cast<const int64_t *>(kind_p));
  const double alpha = *static_cast<const double *>(alpha_p);
  const int64_t n = elements(x) / (FAM == VOIGT ? 6 : 9);
  cudaError_t err = cudaSuccess;
  const int res = eval_t(FAM, kind, alpha, n, static_cast<const T *>(x->data), p, st, &err);
  return launch_error(api, res, err);
}

// adjoints: arguments A, W, V ((..., 3, 3); W or V with no elements when not given), attributes kind, alpha and
// outputs (bits 1 F, 2 J^T W, 4 J V, 8 W.H.V), one result per set bit in that order; as smf_cuda_adjoint /
// gmf_cuda_adjoint (T = double) or their FP32 forms
int adjoint_t(bool gen, int kind, double al, int64_t n, const double *A, const double *W, const double *V, double **o,
              cudaStream_t st) {
  return gen ? gmf_cuda_adjoint(kind, al, n, A, W, V, o[0], o[1], o[2], o[3], st)
             : smf_cuda_adjoint(kind, al, n, A, W, V, o[0], o[1], o[2], o[3], st);
}
int adjoint_t(bool gen, int kind, double al, int64_t n, const float *A, const float *W, const float *V, float **o,
              cudaStream_t st) {
  return gen ? gmf_cuda_adjoint_f32(kind, al, n, A, W, V, o[0], o[1], o[2], o[3], st)
             : smf_cuda_adjoint_f32(kind, al, n, A, W, V, o[0], o[1], o[2], o[3], st);
}

template <bool GEN, typename T>
void *handle_adjoint(mfx_call_frame *cf) {
  const mfx_api *api = cf->api;
  bool done;
  if (void *r = frame_checks(cf, 3, 3, &done); done) return r;
  constexpr int DT = dtype_of<T>();
  cudaStream_t st;
  if (void *e = get_stream(cf, &st)) return e;
  std::string why;
  const mfx_buffer *in[3];
  for (int i = 0; i < 3; i++)
    in[i] = typed_buffer(cf->args.types[i], cf->args.args[i], MFX_ARG_BUFFER, DT, "argument", why);
  const void *kind_p = scalar_attr(cf->attrs, "kind", MFX_DT_S64, why);
  const void *alpha_p = scalar_attr(cf->attrs, "alpha", MFX_DT_F64, why);
  const void *outs_p = scalar_attr(cf->attrs, "outputs", MFX_DT_S64, why);
  if (!why.empty()) return invalid(api, "Failed to decode all FFI handler operands: " + why);
  const mfx_buffer *A = in[0];
  const int64_t r = A->rank;
  if (!(r >= 2 && A->dims[r - 1] == 3 && A->dims[r - 2] == 3))
    return invalid(api, "matfun: expected matrices of shape (..., 3, 3)");
  const int64_t cnt = elements(A);
  const T *dirs[2] = {nullptr, nullptr};
  for (int i = 1; i < 3; i++) {
    const int64_t c = elements(in[i]);
    if (c != 0 && c != cnt) return invalid(api, "matfun: W and V must have the shape of A (or no elements)");
    dirs[i - 1] = c ? static_cast<const T *>(in[i]->data) : nullptr;
  }
  const int64_t outs = *static_cast<const int64_t *>(outs_p);
  if (outs < 1 || outs > 15) return invalid(api, "matfun: outputs must select some of F, J^T W, J V, W.H.V");
  int want = 0;
  for (int b = 0; b < 4; b++) want += (int)((outs >> b) & 1);
  if (cf->rets.size != want) return invalid(api, "matfun: one result per selected output expected");
  T *o[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int b = 0, i = 0; b < 4; b++) {
    if (!((outs >> b) & 1)) continue;
    const mfx_buffer *rb = typed_buffer(cf->rets.types[i], cf->rets.rets[i], MFX_RET_BUFFER, DT, "result", why);
    if (rb == nullptr) return invalid(api, "Failed to decode result " + std::to_string(i) + ": " + why);
    if (elements(rb) != cnt) return invalid(api, "matfun: every result has the shape of A");
    o[b] = static_cast<T *>(rb->data);
    i++;
  }
  const int kind = clamp_kind(*static_cast<const int64_t *>(kind_p));
  const double alpha = *static_cast<const double *>(alpha_p);
  if (cnt == 0) return nullptr;  // no matrices: nothing to launch (W and V cannot be told apart from absent)
  const int res = adjoint_t(GEN, kind, alpha, cnt / 9, static_cast<const T *>(A->data), dirs[0], dirs[1], o, st);
  return launch_error(api, res, cudaPeekAtLastError());
}

// A -> the selected ones of F = f(A), G = J^T F, K = J^T J + F : H (gmf_cuda_tangent; attribute `outputs`: bit 0 F,
// bit 1 G, bit 2 K, which is required), results in that order; F and G of A's shape, K of 9 times its elements
void *handle_tangent(mfx_call_frame *cf) {
  const mfx_api *api = cf->api;
  bool done;
  if (void *r = frame_checks(cf, 1, 3, &done); done) return r;
  cudaStream_t st;
  if (void *e = get_stream(cf, &st)) return e;
  std::string why;
  const mfx_buffer *A = typed_buffer(cf->args.types[0], cf->args.args[0], MFX_ARG_BUFFER, MFX_DT_F64, "argument", why);
  const void *kind_p = scalar_attr(cf->attrs, "kind", MFX_DT_S64, why);
  const void *alpha_p = scalar_attr(cf->attrs, "alpha", MFX_DT_F64, why);
  const void *outs_p = scalar_attr(cf->attrs, "outputs", MFX_DT_S64, why);
  if (!why.empty()) return invalid(api, "Failed to decode all FFI handler operands: " + why);
  const int64_t r = A->rank;
  if (!(r >= 2 && A->dims[r - 1] == 3 && A->dims[r - 2] == 3))
    return invalid(api, "matfun: expected matrices of shape (..., 3, 3)");
  const int64_t cnt = elements(A);
  const int64_t outs = *static_cast<const int64_t *>(outs_p);
  if (outs < 4 || outs > 7) return invalid(api, "matfun: outputs must select K and optionally F, G");
  const int want = 1 + (int)(outs & 1) + (int)((outs >> 1) & 1);
  if (cf->rets.size != want) return invalid(api, "matfun: one result per selected output expected");
  double *o[3] = {nullptr, nullptr, nullptr};
  for (int b = 0, i = 0; b < 3; b++) {
    if (!((outs >> b) & 1)) continue;
    const mfx_buffer *rb =
        typed_buffer(cf->rets.types[i], cf->rets.rets[i], MFX_RET_BUFFER, MFX_DT_F64, "result", why);
    if (rb == nullptr) return invalid(api, "Failed to decode result " + std::to_string(i) + ": " + why);
    if (elements(rb) != (b == 2 ? 9 * cnt : cnt)) return invalid(api, "matfun: F and G have A's shape, K 9 times it");
    o[b] = static_cast<double *>(rb->data);
    i++;
  }
  const int kind = clamp_kind(*static_cast<const int64_t *>(kind_p));
  const double alpha = *static_cast<const double *>(alpha_p);
  if (cnt == 0) return nullptr;
  const int res = gmf_cuda_tangent(kind, alpha, cnt / 9, static_cast<const double *>(A->data), o[0], o[1], o[2], st);
  return launch_error(api, res, cudaPeekAtLastError());
}

}  // namespace

#define MF_FFI_HANDLER(name, fam, T) \
  extern "C" void *name(void *call_frame) { return handle<fam, T>(static_cast<mfx_call_frame *>(call_frame)); }

MF_FFI_HANDLER(SmfValueCuda, VOIGT, double)
MF_FFI_HANDLER(SmfValueJacCuda, VOIGT, double)
MF_FFI_HANDLER(SmfValueJacHessCuda, VOIGT, double)
MF_FFI_HANDLER(SmfMatrixValueCuda, MATRIX, double)
MF_FFI_HANDLER(SmfMatrixValueJacCuda, MATRIX, double)
MF_FFI_HANDLER(SmfMatrixValueJacHessCuda, MATRIX, double)
MF_FFI_HANDLER(GmfValueCuda, GENERAL, double)
MF_FFI_HANDLER(GmfValueJacCuda, GENERAL, double)
MF_FFI_HANDLER(GmfValueJacHessCuda, GENERAL, double)

// additions (no counterpart in the reference): the FP32 forms and the adjoints
MF_FFI_HANDLER(SmfValueF32Cuda, VOIGT, float)
MF_FFI_HANDLER(SmfMatrixValueF32Cuda, MATRIX, float)
MF_FFI_HANDLER(GmfValueF32Cuda, GENERAL, float)

#define MF_FFI_ADJOINT(name, gen, T) \
  extern "C" void *name(void *call_frame) { return handle_adjoint<gen, T>(static_cast<mfx_call_frame *>(call_frame)); }

MF_FFI_ADJOINT(SmfAdjointCuda, false, double)
MF_FFI_ADJOINT(GmfAdjointCuda, true, double)
MF_FFI_ADJOINT(SmfAdjointF32Cuda, false, float)
MF_FFI_ADJOINT(GmfAdjointF32Cuda, true, float)

extern "C" void *GmfTangentCuda(void *call_frame) { return handle_tangent(static_cast<mfx_call_frame *>(call_frame)); }

extern "C" int smf_xla_ffi_api_version(void) { return MFX_API_MAJOR * 1000 + MFX_API_MINOR; }

// xla_ffi.cu -- the XLA FFI custom-call handlers that matfun.jax registers for the CUDA platform
// (cuda/src/matfun_cuda.cu:209-265; python/src/matfun/jax.py:66-87 binds them by name and checks
// smf_xla_ffi_api_version): SmfValueCuda ... GmfValueJacHessCuda.
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

// an F64 buffer (argument or result), or nullptr with the reason in why
const mfx_buffer *f64_buffer(int32_t type, void *p, int expected_type, const char *what, std::string &why) {
  const mfx_buffer *b = static_cast<const mfx_buffer *>(p);
  if (type != expected_type || b == nullptr) {
    why += std::string(why.empty() ? "" : "; ") + "wrong " + what + " type: expected a buffer";
    return nullptr;
  }
  if (b->dtype != MFX_DT_F64) {
    why += std::string(why.empty() ? "" : "; ") + "wrong " + what + " dtype: expected F64 but got " +
           std::to_string(b->dtype);
    return nullptr;
  }
  return b;
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

template <int FAM>
void *handle(mfx_call_frame *cf) {
  const mfx_api *api = cf->api;
  if (cf->struct_size != MFX_CALL_FRAME_SIZE)
    return invalid(api, "Unexpected XLA_FFI_CallFrame size: expected " + std::to_string(MFX_CALL_FRAME_SIZE) +
                            " got " + std::to_string(cf->struct_size) + ". Check installed software versions.");
  if (cf->extension_start != nullptr && cf->extension_start->type == MFX_EXT_METADATA)
    return metadata(api, reinterpret_cast<mfx_metadata_ext *>(cf->extension_start));
  if (cf->stage != MFX_STAGE_EXECUTE)
    return invalid(api, "Wrong execution stage: expected `3` but got `" + std::to_string(cf->stage) + "`");
  if (cf->args.size != 1)
    return invalid(api, "Wrong number of arguments: expected 1 but got " + std::to_string(cf->args.size));
  if (cf->attrs.size != 2)
    return invalid(api, "Wrong number of attributes: expected 2 but got " + std::to_string(cf->attrs.size));

  // operands, in the order of the binding: XLA's stream, x, (the results), kind, alpha
  mfx_stream_get_args sa;
  sa.struct_size = MFX_STREAM_GET_ARGS_SIZE;
  sa.extension_start = nullptr;
  sa.ctx = cf->ctx;
  sa.stream = nullptr;
  if (void *e = api->stream_get(&sa)) return e;
  std::string why;
  const mfx_buffer *x = f64_buffer(cf->args.types[0], cf->args.args[0], MFX_ARG_BUFFER, "argument", why);
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
  double *p[3] = {nullptr, nullptr, nullptr};
  for (int64_t i = 0; i < cf->rets.size; i++) {
    const mfx_buffer *b = f64_buffer(cf->rets.types[i], cf->rets.rets[i], MFX_RET_BUFFER, "result", why);
    if (b == nullptr) return invalid(api, "Failed to decode result " + std::to_string(i) + ": " + why);
    p[i] = static_cast<double *>(b->data);
  }
  int64_t count = 1;
  for (int64_t d = 0; d < r; d++) count *= x->dims[d];
  const int64_t kind64 = *static_cast<const int64_t *>(kind_p);
  const int kind = (int)std::min<int64_t>(std::max<int64_t>(kind64, -1), SMF_SQRT + 1);  // out of int range: invalid
  const double alpha = *static_cast<const double *>(alpha_p);
  const int64_t n = count / (FAM == VOIGT ? 6 : 9);
  cudaError_t err = cudaSuccess;
  const int res = mf::eval_f64(FAM, kind, alpha, n, static_cast<const double *>(x->data), p[0], p[1], p[2],
                               (cudaStream_t)sa.stream, &err);
  if (res == -1) return invalid(api, "matfun: invalid kind or alpha");
  if (res != 0) return make_error(api, MFX_ERR_INTERNAL, std::string("matfun: CUDA launch failed: ") +
                                                             (err == cudaSuccess ? "grid limit" : cudaGetErrorString(err)));
  return nullptr;
}

}  // namespace

#define MF_FFI_HANDLER(name, fam) \
  extern "C" void *name(void *call_frame) { return handle<fam>(static_cast<mfx_call_frame *>(call_frame)); }

MF_FFI_HANDLER(SmfValueCuda, VOIGT)
MF_FFI_HANDLER(SmfValueJacCuda, VOIGT)
MF_FFI_HANDLER(SmfValueJacHessCuda, VOIGT)
MF_FFI_HANDLER(SmfMatrixValueCuda, MATRIX)
MF_FFI_HANDLER(SmfMatrixValueJacCuda, MATRIX)
MF_FFI_HANDLER(SmfMatrixValueJacHessCuda, MATRIX)
MF_FFI_HANDLER(GmfValueCuda, GENERAL)
MF_FFI_HANDLER(GmfValueJacCuda, GENERAL)
MF_FFI_HANDLER(GmfValueJacHessCuda, GENERAL)

extern "C" int smf_xla_ffi_api_version(void) { return MFX_API_MAJOR * 1000 + MFX_API_MINOR; }

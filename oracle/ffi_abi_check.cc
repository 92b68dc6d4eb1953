// Test infrastructure (oracle/Makefile.ref, target ffi-abi): static checks that matfun_gb300/csrc/xla_ffi_abi.h
// declares the XLA FFI C API 0.1 structures with the layout of the XLA FFI header vendored by the reference
// (third_party/xla_ffi/include/xla/ffi/api/c_api.h).  Compiled with -fsyntax-only; nothing is linked or run.
#include <cstddef>

#include "xla/ffi/api/c_api.h"
#include "../matfun_gb300/csrc/xla_ffi_abi.h"

#define SAME_SIZE(a, b) static_assert(sizeof(a) == sizeof(b), "size of " #a)
#define SAME_FIELD(a, fa, b, fb) \
  static_assert(offsetof(a, fa) == offsetof(b, fb) && sizeof(((a *)0)->fa) == sizeof(((b *)0)->fb), #a "." #fa)

#define SAME_VALUE(a, b) static_assert((long)(a) == (long)(b), #a)

SAME_VALUE(XLA_FFI_API_MAJOR, MFX_API_MAJOR);
SAME_VALUE(XLA_FFI_API_MINOR, MFX_API_MINOR);
SAME_VALUE(XLA_FFI_Extension_Metadata, MFX_EXT_METADATA);
SAME_VALUE(XLA_FFI_Error_Code_INVALID_ARGUMENT, MFX_ERR_INVALID_ARGUMENT);
SAME_VALUE(XLA_FFI_Error_Code_INTERNAL, MFX_ERR_INTERNAL);
SAME_VALUE(XLA_FFI_DataType_S64, MFX_DT_S64);
SAME_VALUE(XLA_FFI_DataType_F32, MFX_DT_F32);
SAME_VALUE(XLA_FFI_DataType_F64, MFX_DT_F64);
SAME_VALUE(XLA_FFI_ArgType_BUFFER, MFX_ARG_BUFFER);
SAME_VALUE(XLA_FFI_RetType_BUFFER, MFX_RET_BUFFER);
SAME_VALUE(XLA_FFI_AttrType_SCALAR, MFX_ATTR_SCALAR);
SAME_VALUE(XLA_FFI_ExecutionStage_EXECUTE, MFX_STAGE_EXECUTE);
static_assert(sizeof(XLA_FFI_DataType) == sizeof(int32_t) && sizeof(XLA_FFI_ArgType) == sizeof(int32_t) &&
              sizeof(XLA_FFI_AttrType) == sizeof(int32_t) && sizeof(XLA_FFI_ExecutionStage) == sizeof(int32_t),
              "enumerations are 32-bit");

SAME_SIZE(XLA_FFI_Extension_Base, mfx_ext);
SAME_FIELD(XLA_FFI_Extension_Base, type, mfx_ext, type);
SAME_FIELD(XLA_FFI_Extension_Base, next, mfx_ext, next);
SAME_SIZE(XLA_FFI_Api_Version, mfx_api_version);
SAME_FIELD(XLA_FFI_Api_Version, major_version, mfx_api_version, major_version);
SAME_FIELD(XLA_FFI_Api_Version, minor_version, mfx_api_version, minor_version);
SAME_SIZE(XLA_FFI_Error_Create_Args, mfx_error_create_args);
SAME_FIELD(XLA_FFI_Error_Create_Args, message, mfx_error_create_args, message);
SAME_FIELD(XLA_FFI_Error_Create_Args, errc, mfx_error_create_args, errc);
SAME_SIZE(XLA_FFI_Buffer, mfx_buffer);
SAME_FIELD(XLA_FFI_Buffer, dtype, mfx_buffer, dtype);
SAME_FIELD(XLA_FFI_Buffer, data, mfx_buffer, data);
SAME_FIELD(XLA_FFI_Buffer, rank, mfx_buffer, rank);
SAME_FIELD(XLA_FFI_Buffer, dims, mfx_buffer, dims);
SAME_SIZE(XLA_FFI_ByteSpan, mfx_bytespan);
SAME_FIELD(XLA_FFI_ByteSpan, len, mfx_bytespan, len);
SAME_SIZE(XLA_FFI_Scalar, mfx_scalar);
SAME_FIELD(XLA_FFI_Scalar, value, mfx_scalar, value);
SAME_SIZE(XLA_FFI_Args, mfx_args);
SAME_FIELD(XLA_FFI_Args, size, mfx_args, size);
SAME_FIELD(XLA_FFI_Args, types, mfx_args, types);
SAME_FIELD(XLA_FFI_Args, args, mfx_args, args);
SAME_SIZE(XLA_FFI_Rets, mfx_rets);
SAME_FIELD(XLA_FFI_Rets, rets, mfx_rets, rets);
SAME_SIZE(XLA_FFI_Attrs, mfx_attrs);
SAME_FIELD(XLA_FFI_Attrs, types, mfx_attrs, types);
SAME_FIELD(XLA_FFI_Attrs, names, mfx_attrs, names);
SAME_FIELD(XLA_FFI_Attrs, attrs, mfx_attrs, attrs);
SAME_SIZE(XLA_FFI_CallFrame, mfx_call_frame);
SAME_FIELD(XLA_FFI_CallFrame, api, mfx_call_frame, api);
SAME_FIELD(XLA_FFI_CallFrame, ctx, mfx_call_frame, ctx);
SAME_FIELD(XLA_FFI_CallFrame, stage, mfx_call_frame, stage);
SAME_FIELD(XLA_FFI_CallFrame, args, mfx_call_frame, args);
SAME_FIELD(XLA_FFI_CallFrame, rets, mfx_call_frame, rets);
SAME_FIELD(XLA_FFI_CallFrame, attrs, mfx_call_frame, attrs);
SAME_FIELD(XLA_FFI_CallFrame, future, mfx_call_frame, future);
SAME_SIZE(XLA_FFI_Stream_Get_Args, mfx_stream_get_args);
SAME_FIELD(XLA_FFI_Stream_Get_Args, ctx, mfx_stream_get_args, ctx);
SAME_FIELD(XLA_FFI_Stream_Get_Args, stream, mfx_stream_get_args, stream);
SAME_SIZE(XLA_FFI_Metadata, mfx_metadata);
SAME_FIELD(XLA_FFI_Metadata, api_version, mfx_metadata, api_version);
SAME_FIELD(XLA_FFI_Metadata, traits, mfx_metadata, traits);
SAME_SIZE(XLA_FFI_Metadata_Extension, mfx_metadata_ext);
SAME_FIELD(XLA_FFI_Metadata_Extension, metadata, mfx_metadata_ext, metadata);
SAME_FIELD(XLA_FFI_Api, api_version, mfx_api, api_version);
SAME_FIELD(XLA_FFI_Api, internal_api, mfx_api, internal_api);
SAME_FIELD(XLA_FFI_Api, XLA_FFI_Error_Create, mfx_api, error_create);
SAME_FIELD(XLA_FFI_Api, XLA_FFI_Stream_Get, mfx_api, stream_get);

static_assert(XLA_FFI_CallFrame_STRUCT_SIZE == MFX_CALL_FRAME_SIZE, "call frame size macro");
static_assert(XLA_FFI_Error_Create_Args_STRUCT_SIZE == MFX_ERROR_CREATE_ARGS_SIZE, "error args size macro");
static_assert(XLA_FFI_Stream_Get_Args_STRUCT_SIZE == MFX_STREAM_GET_ARGS_SIZE, "stream args size macro");
static_assert(XLA_FFI_Api_Version_STRUCT_SIZE == MFX_API_VERSION_SIZE, "version size macro");
static_assert(XLA_FFI_Metadata_STRUCT_SIZE == MFX_METADATA_SIZE, "metadata size macro");
static_assert(XLA_FFI_Metadata_Extension_STRUCT_SIZE == MFX_METADATA_EXT_SIZE, "metadata extension size macro");

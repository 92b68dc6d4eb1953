/* xla_ffi_abi.h -- the part of the XLA FFI C API (API version 0.1) that the custom-call handlers of this library
 * read: the call frame, its argument / result / attribute arrays, buffers, scalar attributes, the metadata query and
 * the two API functions used (error creation, stream lookup).
 *
 * These are this project's own declarations of a published binary interface (OpenXLA, xla/ffi/api/c_api.h); field
 * order, types and sizes have to be those of the interface, the names are this project's (prefix mfx_).  Enumerated
 * values are 32-bit integers, as the C enums of the interface are.  The handlers need no XLA or JAX headers to build.
 */
#ifndef MATFUN_XLA_FFI_ABI_H
#define MATFUN_XLA_FFI_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFX_API_MAJOR 0
#define MFX_API_MINOR 1

enum {
  MFX_EXT_METADATA = 1,
  MFX_ERR_INVALID_ARGUMENT = 3,
  MFX_ERR_INTERNAL = 13,
  MFX_DT_S64 = 5,
  MFX_DT_F32 = 11,
  MFX_DT_F64 = 12,
  MFX_ARG_BUFFER = 1,
  MFX_RET_BUFFER = 1,
  MFX_ATTR_SCALAR = 3,
  MFX_STAGE_EXECUTE = 3
};

typedef struct mfx_ext {
  size_t struct_size;
  int32_t type;
  struct mfx_ext *next;
} mfx_ext;

typedef struct mfx_api_version {
  size_t struct_size;
  mfx_ext *extension_start;
  int32_t major_version;
  int32_t minor_version;
} mfx_api_version;

typedef struct mfx_error_create_args {
  size_t struct_size;
  mfx_ext *extension_start;
  const char *message;
  int32_t errc;
} mfx_error_create_args;

typedef struct mfx_buffer {
  size_t struct_size;
  mfx_ext *extension_start;
  int32_t dtype;
  void *data;
  int64_t rank;
  int64_t *dims;
} mfx_buffer;

typedef struct mfx_bytespan {
  const char *ptr;
  size_t len;
} mfx_bytespan;

typedef struct mfx_scalar {
  int32_t dtype;
  void *value;
} mfx_scalar;

typedef struct mfx_args {
  size_t struct_size;
  mfx_ext *extension_start;
  int64_t size;
  int32_t *types;
  void **args;
} mfx_args;

typedef struct mfx_rets {
  size_t struct_size;
  mfx_ext *extension_start;
  int64_t size;
  int32_t *types;
  void **rets;
} mfx_rets;

typedef struct mfx_attrs {
  size_t struct_size;
  mfx_ext *extension_start;
  int64_t size;
  int32_t *types;
  mfx_bytespan **names;  /* sorted by name */
  void **attrs;
} mfx_attrs;

typedef struct mfx_api mfx_api;

typedef struct mfx_call_frame {
  size_t struct_size;
  mfx_ext *extension_start;
  const mfx_api *api;
  void *ctx;
  int32_t stage;
  mfx_args args;
  mfx_rets rets;
  mfx_attrs attrs;
  void *future;
} mfx_call_frame;

typedef struct mfx_stream_get_args {
  size_t struct_size;
  mfx_ext *extension_start;
  void *ctx;
  void *stream;
} mfx_stream_get_args;

typedef struct mfx_metadata {
  size_t struct_size;
  mfx_api_version api_version;
  uint32_t traits;
} mfx_metadata;

typedef struct mfx_metadata_ext {
  mfx_ext extension_base;
  mfx_metadata *metadata;
} mfx_metadata_ext;

struct mfx_api {
  size_t struct_size;
  mfx_ext *extension_start;
  mfx_api_version api_version;
  void *internal_api;
  void *(*error_create)(mfx_error_create_args *);
  void (*error_get_message)(void *);
  void (*error_destroy)(void *);
  void *(*handler_register)(void *);
  void *(*stream_get)(mfx_stream_get_args *);
  /* further functions of the interface are not used */
};

/* the interface's structure sizes: offset of the last field of the version + its size */
#define MFX_SIZE_UPTO(type, field) (offsetof(type, field) + sizeof(((type *)0)->field))
#define MFX_CALL_FRAME_SIZE MFX_SIZE_UPTO(mfx_call_frame, attrs)
#define MFX_ERROR_CREATE_ARGS_SIZE MFX_SIZE_UPTO(mfx_error_create_args, errc)
#define MFX_STREAM_GET_ARGS_SIZE MFX_SIZE_UPTO(mfx_stream_get_args, stream)
#define MFX_API_VERSION_SIZE MFX_SIZE_UPTO(mfx_api_version, minor_version)
#define MFX_METADATA_SIZE MFX_SIZE_UPTO(mfx_metadata, traits)
#define MFX_METADATA_EXT_SIZE MFX_SIZE_UPTO(mfx_metadata_ext, metadata)

#ifdef __cplusplus
}
#endif

#endif

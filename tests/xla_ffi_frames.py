"""Test infrastructure: XLA FFI call frames built with ctypes, so that the custom-call handlers of libmatfun_cuda can be
called the way XLA calls them (one call frame per custom call; XLA FFI C API 0.1, the layout of
matfun_gb300/csrc/xla_ffi_abi.h).  A fake API object records the errors the handler creates and hands out the stream."""
import ctypes as C

DT_S64, DT_F32, DT_F64 = 5, 11, 12
ARG_BUFFER = RET_BUFFER = 1
ATTR_SCALAR = 3
STAGE_EXECUTE = 3
EXT_METADATA = 1
ERR_INVALID_ARGUMENT, ERR_INTERNAL = 3, 13


class Ext(C.Structure):
    pass


Ext._fields_ = [("struct_size", C.c_size_t), ("type", C.c_int32), ("next", C.POINTER(Ext))]


class ApiVersion(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("major_version", C.c_int32),
                ("minor_version", C.c_int32)]


class ErrorCreateArgs(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("message", C.c_char_p),
                ("errc", C.c_int32)]


class Buffer(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("dtype", C.c_int32),
                ("data", C.c_void_p), ("rank", C.c_int64), ("dims", C.POINTER(C.c_int64))]


class ByteSpan(C.Structure):
    _fields_ = [("ptr", C.c_char_p), ("len", C.c_size_t)]


class Scalar(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("value", C.c_void_p)]


class Args(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("size", C.c_int64),
                ("types", C.POINTER(C.c_int32)), ("args", C.POINTER(C.c_void_p))]


class Attrs(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("size", C.c_int64),
                ("types", C.POINTER(C.c_int32)), ("names", C.POINTER(C.POINTER(ByteSpan))),
                ("attrs", C.POINTER(C.c_void_p))]


class StreamGetArgs(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("ctx", C.c_void_p),
                ("stream", C.c_void_p)]


class Metadata(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("api_version", ApiVersion), ("traits", C.c_uint32)]


class MetadataExt(C.Structure):
    _fields_ = [("extension_base", Ext), ("metadata", C.POINTER(Metadata))]


ERROR_CREATE = C.CFUNCTYPE(C.c_void_p, C.POINTER(ErrorCreateArgs))
STREAM_GET = C.CFUNCTYPE(C.c_void_p, C.POINTER(StreamGetArgs))


class Api(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.c_void_p), ("api_version", ApiVersion),
                ("internal_api", C.c_void_p), ("error_create", ERROR_CREATE), ("error_get_message", C.c_void_p),
                ("error_destroy", C.c_void_p), ("handler_register", C.c_void_p), ("stream_get", STREAM_GET)]


class CallFrame(C.Structure):
    _fields_ = [("struct_size", C.c_size_t), ("extension_start", C.POINTER(Ext)), ("api", C.POINTER(Api)),
                ("ctx", C.c_void_p), ("stage", C.c_int32), ("args", Args), ("rets", Args), ("attrs", Attrs),
                ("future", C.c_void_p)]


CALL_FRAME_SIZE = CallFrame.attrs.offset + C.sizeof(Attrs)


class FakeXla:
    """the API object of one XLA instance: records created errors, returns `stream` from the stream lookup"""

    def __init__(self, stream=0):
        self.errors = []
        self.stream = stream
        self._ec = ERROR_CREATE(self._error_create)
        self._sg = STREAM_GET(self._stream_get)
        self.api = Api(struct_size=C.sizeof(Api), error_create=self._ec, stream_get=self._sg)
        self.api.api_version = ApiVersion(C.sizeof(ApiVersion), None, 0, 1)

    def _error_create(self, a):
        self.errors.append((a.contents.errc, a.contents.message.decode()))
        return len(self.errors)  # a distinct non-NULL handle per error

    def _stream_get(self, a):
        a.contents.stream = self.stream
        return None


def _buffer(dtype, ptr, dims, keep):
    d = (C.c_int64 * max(len(dims), 1))(*dims)
    b = Buffer(struct_size=C.sizeof(Buffer), dtype=dtype, data=ptr, rank=len(dims),
               dims=C.cast(d, C.POINTER(C.c_int64)))
    keep += [d, b]
    return b


def frame(xla, x, rets, attrs, stage=STAGE_EXECUTE, struct_size=None, arg_types=None, ret_types=None):
    """a call frame: x = (dtype, device pointer, dims); rets = [(dtype, pointer, dims)]; attrs = {name: (attr type,
    dtype, ctypes value)} (sorted by name, as XLA passes them).  Returns (frame, keep-alive list)."""
    keep = []
    xs = [x] if x is not None else []
    bufs = [_buffer(*b, keep) for b in xs]
    at = (C.c_int32 * max(len(bufs), 1))(*(arg_types or [ARG_BUFFER] * len(bufs)))
    ap = (C.c_void_p * max(len(bufs), 1))(*[C.addressof(b) for b in bufs])
    rb = [_buffer(*b, keep) for b in rets]
    rt = (C.c_int32 * max(len(rb), 1))(*(ret_types or [RET_BUFFER] * len(rb)))
    rp = (C.c_void_p * max(len(rb), 1))(*[C.addressof(b) for b in rb])
    names = sorted(attrs)
    spans, scal, vals = [], [], []
    for nm in names:
        atype, dtype, val = attrs[nm]
        enc = nm.encode()
        spans.append(ByteSpan(enc, len(enc)))
        vals.append(val)
        scal.append(Scalar(dtype, C.cast(C.pointer(val), C.c_void_p)))
    sp = (C.POINTER(ByteSpan) * max(len(names), 1))(*[C.pointer(s) for s in spans])
    aty = (C.c_int32 * max(len(names), 1))(*[attrs[nm][0] for nm in names])
    avp = (C.c_void_p * max(len(names), 1))(*[C.addressof(s) for s in scal])
    keep += [at, ap, rt, rp, spans, scal, vals, sp, aty, avp, xla]
    cf = CallFrame(struct_size=struct_size if struct_size is not None else CALL_FRAME_SIZE,
                   api=C.pointer(xla.api), stage=stage)
    cf.args = Args(C.sizeof(Args), None, len(bufs), C.cast(at, C.POINTER(C.c_int32)), C.cast(ap, C.POINTER(C.c_void_p)))
    cf.rets = Args(C.sizeof(Args), None, len(rb), C.cast(rt, C.POINTER(C.c_int32)), C.cast(rp, C.POINTER(C.c_void_p)))
    cf.attrs = Attrs(C.sizeof(Attrs), None, len(names), C.cast(aty, C.POINTER(C.c_int32)),
                     C.cast(sp, C.POINTER(C.POINTER(ByteSpan))), C.cast(avp, C.POINTER(C.c_void_p)))
    return cf, keep


def std_attrs(kind, alpha):
    return {"kind": (ATTR_SCALAR, DT_S64, C.c_int64(kind)), "alpha": (ATTR_SCALAR, DT_F64, C.c_double(alpha))}


def frame3(xla, args, rets, attrs):
    """a call frame with several arguments (the adjoint handlers: A, W, V)"""
    cf, keep = frame(xla, args[0], rets, attrs)
    bufs = [_buffer(*a, keep) for a in args]
    at = (C.c_int32 * len(bufs))(*([ARG_BUFFER] * len(bufs)))
    ap = (C.c_void_p * len(bufs))(*[C.addressof(b) for b in bufs])
    keep += [at, ap]
    cf.args = Args(C.sizeof(Args), None, len(bufs), C.cast(at, C.POINTER(C.c_int32)), C.cast(ap, C.POINTER(C.c_void_p)))
    return cf, keep


def adjoint_attrs(kind, alpha, outputs):
    return {**std_attrs(kind, alpha), "outputs": (ATTR_SCALAR, DT_S64, C.c_int64(outputs))}


HANDLERS = {"voigt": ("SmfValueCuda", "SmfValueJacCuda", "SmfValueJacHessCuda"),
            "matrix": ("SmfMatrixValueCuda", "SmfMatrixValueJacCuda", "SmfMatrixValueJacHessCuda"),
            "general": ("GmfValueCuda", "GmfValueJacCuda", "GmfValueJacHessCuda")}


def handler(lib, name):
    fn = getattr(lib, name)
    fn.restype = C.c_void_p
    fn.argtypes = [C.c_void_p]
    return fn

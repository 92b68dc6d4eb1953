"""ctypes binding of libmatfun_cuda.so (the C ABI of include/matfun_cuda.h).

The library is built in-tree (matfun_gb300/build.py); MATFUN_CUDA_LIB overrides the path, as for the reference's
JAX plugin (python/src/matfun/jax.py:100-103).  There is no CPU fallback: loading fails loudly when the library is
missing.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None

KINDS = {"exp": 0, "log": 1, "pow": 2, "sqrt": 3}

class Request(ctypes.Structure):
    """mf_request of include/matfun_cuda.h"""
    _fields_ = [("family", ctypes.c_int32), ("kind", ctypes.c_int32), ("order", ctypes.c_int32),
                ("dtype", ctypes.c_int32), ("alpha", ctypes.c_double), ("n", ctypes.c_int64),
                ("x", ctypes.c_void_p), ("F", ctypes.c_void_p), ("J", ctypes.c_void_p), ("H", ctypes.c_void_p)]


# exported symbol -> (restype, argtypes)
_EVAL = [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 5
SIGNATURES = {
    "smf_cuda_eval": (ctypes.c_int, _EVAL),
    "smf_cuda_eval_matrix": (ctypes.c_int, _EVAL),
    "gmf_cuda_eval": (ctypes.c_int, _EVAL),
    "smf_cuda_eval_f32": (ctypes.c_int, _EVAL),
    "smf_cuda_eval_matrix_f32": (ctypes.c_int, _EVAL),
    "gmf_cuda_eval_f32": (ctypes.c_int, _EVAL),
    "smf_cuda_adjoint": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 8),
    "gmf_cuda_adjoint": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 8),
    "smf_cuda_adjoint_f32": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 8),
    "gmf_cuda_adjoint_f32": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 8),
    "gmf_cuda_tangent": (ctypes.c_int, _EVAL),
    "smf_cuda_eval_host": (ctypes.c_int, _EVAL[:-1]),
    "smf_cuda_eval_matrix_host": (ctypes.c_int, _EVAL[:-1]),
    "gmf_cuda_eval_host": (ctypes.c_int, _EVAL[:-1]),
    "matfun_cuda_fp64_peak": (ctypes.c_int, [ctypes.c_void_p]),
    "matfun_cuda_fp32_peak": (ctypes.c_int, [ctypes.c_void_p]),
    "matfun_cuda_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "matfun_cuda_batched_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "matfun_cuda_batched_plan": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "matfun_cuda_batched_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "matfun_cuda_batched_free": (ctypes.c_int, [ctypes.c_void_p]),
    "matfun_cuda_batched_tune": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "matfun_cuda_batched_tune_tiles": (ctypes.c_int, [ctypes.c_int]),
    "matfun_cuda_smf_f32_tune": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "matfun_cuda_version": (ctypes.c_char_p, []),
}


def library_path():
    return os.environ.get("MATFUN_CUDA_LIB") or os.path.join(HERE, "libmatfun_cuda.so")


def load():
    """the loaded library (raises OSError if it is missing: build it with matfun_gb300.build)"""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise OSError(f"libmatfun_cuda not found at {path}; run `python -m matfun_gb300.build`")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        _lib = lib
    return _lib

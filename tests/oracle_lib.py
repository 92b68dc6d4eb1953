"""NumPy driver of the CPU oracle (oracle/liboracle.so, a scalar C restatement of the reference algorithm) and, where
it was built, of the reference's own CPU library (oracle/_ref/libmatfun_ref.so).  Test and benchmark infrastructure
only: the checker, never the thing measured as the product.  Same interface as the reference's NumPy API
(python/src/matfun/_capi.py:62-113)."""
import ctypes
import math
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle", "liboracle.so")
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libmatfun_ref.so")
KINDS = {"exp": 0, "log": 1, "pow": 2, "sqrt": 3}
_libs = {}


def _load(path, prefix):
    key = (path, prefix)
    if key not in _libs:
        if not os.path.exists(path):
            raise OSError(f"{path} missing: run __graft_entry__.build()")
        lib = ctypes.CDLL(path)
        fns = {}
        for nm in ("smf_eval", "smf_eval_matrix", "gmf_eval"):
            f = getattr(lib, prefix + nm)
            f.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 4
            f.restype = ctypes.c_int
            fns[nm] = f
        _libs[key] = fns
    return _libs[key]


def oracle():
    return _load(ORACLE, "orc_")


def reference():
    """the reference's compiled CPU library, or None where it could not be built"""
    return _load(REFLIB, "") if os.path.exists(REFLIB) else None


def call(fns, fam, kind, alpha, X, order, nf):
    """raw call: (return code, F, J, H) for n inputs X (n, 6 or 9)"""
    X = np.ascontiguousarray(X, dtype=np.float64)
    n = len(X)
    F = np.empty((n, nf))
    J = np.empty((n, nf * nf)) if order >= 1 else None
    H = np.empty((n, nf ** 3)) if order >= 2 else None
    p = lambda a: None if a is None else a.ctypes.data
    r = fns[fam](kind, float(alpha), n, p(X), p(F), p(J), p(H))
    return r, F, J, H


def _api(fam, kind, A, alpha, order, lib):
    A = np.ascontiguousarray(A, dtype=np.float64)
    if fam == "gmf" or A.shape[-2:] == (3, 3):
        sh, nf, fn = A.shape[:-2], 9, ("gmf_eval" if fam == "gmf" else "smf_eval_matrix")
        shapes = ((3, 3), (3, 3, 3, 3), (3, 3, 3, 3, 3, 3))
    else:
        sh, nf, fn = A.shape[:-1], 6, "smf_eval"
        shapes = ((6,), (6, 6), (6, 6, 6))
    n = math.prod(sh)
    r, F, J, H = call(lib or oracle(), fn, KINDS[kind], alpha or 0.0, A.reshape(n, -1), order, nf)
    out = [x.reshape(sh + s) for x, s in zip((F, J, H), shapes) if x is not None]
    return tuple(out) if order else out[0]


def smf(kind, A, alpha=None, order=0, lib=None):
    return _api("smf", kind, A, alpha, order, lib)


def gmf(kind, A, alpha=None, order=0, lib=None):
    return _api("gmf", kind, A, alpha, order, lib)

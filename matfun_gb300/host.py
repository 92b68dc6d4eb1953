"""NumPy front end on the GPU: matfun.smf / matfun.gmf of the reference (python/src/matfun/_capi.py:62-113) with host
arrays in and out, evaluated through the host-buffer entry points of libmatfun_cuda (smf_cuda_eval_host ...):

    from matfun_gb300 import host
    F, J, H = host.gmf("log", A, order=2)          # A: numpy (..., 3, 3) -> numpy arrays
    F = host.smf("sqrt", V)                         # Voigt vectors (..., 6)

Same arguments, shapes, kinds and errors as the reference's NumPy API: ValueError for an unknown kind, pow without
alpha > 0, an order outside 0..2, a wrong shape, and a non-symmetric matrix given to smf (|A_ij - A_ji| > 1e-8 max
|A_kl|).  pinned=True allocates the outputs page-locked, so that the kernels write them in place over the host link
(the input is then staged page-locked as well); otherwise the batch streams through the GPU in chunks.
"""
import math

import numpy as np

from ._lib import KINDS, load


def _check(kind, alpha, order):
    if kind not in KINDS:
        raise ValueError(f"unknown function {kind!r}, expected one of {sorted(KINDS)}")
    if kind == "pow" and not (alpha is not None and alpha > 0):
        raise ValueError("pow needs an exponent alpha > 0")
    if order not in (0, 1, 2):
        raise ValueError("order must be 0, 1 or 2")


def _alloc(shape, pinned):
    if not pinned:
        return np.empty(shape)
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def _run(fn, kind, alpha, A, sh, shapes, order, pinned):
    if pinned:
        staged = _alloc(A.shape, True)
        staged[...] = A
        A = staged
    out = [_alloc(sh + s, pinned) for s in shapes[:order + 1]] + [None] * (2 - order)
    ptr = lambda a: None if a is None else a.ctypes.data
    r = fn(KINDS[kind], float(alpha or 0.0), math.prod(sh), ptr(A), *map(ptr, out))
    if r == -3:
        raise ValueError("matrix input must be symmetric: |A_ij - A_ji| <= 1e-8 max |A_kl| for each matrix")
    if r != 0:
        raise ValueError(f"the host-buffer entry point returned {r}")
    return tuple(out[:order + 1]) if order else out[0]


def smf(kind, A, alpha=None, order=0, pinned=False):
    """f(A), J, H for symmetric 3x3 matrices A (..., 3, 3) or Voigt vectors (..., 6) on host arrays (the shapes and
    layouts of the reference's matfun.smf)"""
    _check(kind, alpha, order)
    A = np.ascontiguousarray(A, dtype=np.float64)
    lib = load()
    if A.shape[-2:] == (3, 3):
        sh, shapes, fn = A.shape[:-2], ((3, 3), (3, 3, 3, 3), (3, 3, 3, 3, 3, 3)), lib.smf_cuda_eval_matrix_host
    elif A.shape[-1:] == (6,):
        sh, shapes, fn = A.shape[:-1], ((6,), (6, 6), (6, 6, 6)), lib.smf_cuda_eval_host
    else:
        raise ValueError(f"expected matrices (..., 3, 3) or Voigt vectors (..., 6), got shape {A.shape}")
    return _run(fn, kind, alpha, A, sh, shapes, order, pinned)


def gmf(kind, A, alpha=None, order=0, pinned=False):
    """f(A), J, H for general real 3x3 matrices A (..., 3, 3) on host arrays (principal branch; NaN for a matrix with
    a real eigenvalue <= 0 under log, sqrt, pow), the shapes of the reference's matfun.gmf"""
    _check(kind, alpha, order)
    A = np.ascontiguousarray(A, dtype=np.float64)
    if A.shape[-2:] != (3, 3):
        raise ValueError(f"expected matrices (..., 3, 3), got shape {A.shape}")
    shapes = ((3, 3), (3, 3, 3, 3), (3, 3, 3, 3, 3, 3))
    return _run(load().gmf_cuda_eval_host, kind, alpha, A, A.shape[:-2], shapes, order, pinned)

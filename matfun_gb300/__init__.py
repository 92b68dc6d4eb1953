"""matfun_gb300 -- batched 3x3 matrix functions exp, log, sqrt and A^alpha with first and second derivatives on a
GB300 GPU (sm_103a), for symmetric (smf) and general (gmf) matrices.

    F, J, H = matfun_gb300.smf("log", A, order=2)     A: torch float64 CUDA tensor (..., 3, 3) or Voigt (..., 6)
    F, J, H = matfun_gb300.gmf("log", A, order=2)     general matrices (..., 3, 3)

Same shapes, layouts, argument checks and error messages as the reference's NumPy interface
(python/src/matfun/_capi.py:62-113), but the arrays are device tensors and the kernels run on the current CUDA
stream.  smf with matrix input does not detect non-symmetric matrices on the device (their results are NaN), as the
reference's CUDA library (cuda/include/matfun/matfun_cuda.h:1-3).
"""
import math

from ._lib import KINDS, library_path, load

__version__ = "0.1.0"
__all__ = ["smf", "gmf", "library_path", "load", "KINDS"]


def _check(kind, alpha, order):
    if kind not in KINDS:
        raise ValueError(f"unknown function {kind!r}, expected one of {sorted(KINDS)}")
    if kind == "pow" and not (alpha is not None and alpha > 0):
        raise ValueError("pow needs an exponent alpha > 0")
    if order not in (0, 1, 2):
        raise ValueError("order must be 0, 1 or 2")


def _prep(A):
    import torch
    if not isinstance(A, torch.Tensor) or not A.is_cuda:
        raise TypeError("expected a CUDA tensor (the device interface); use the C ABI for host arrays")
    return A.to(torch.float64).contiguous()


def _run(fn, kind, alpha, A, sh, shapes, order):
    import torch
    out = [torch.empty(sh + s, dtype=torch.float64, device=A.device) for s in shapes[:order + 1]]
    out += [None] * (2 - order)
    ptr = lambda t: None if t is None else t.data_ptr()
    n = math.prod(sh)
    stream = torch.cuda.current_stream(A.device).cuda_stream
    with torch.cuda.device(A.device):
        r = fn(KINDS[kind], float(alpha or 0.0), n, ptr(A), *map(ptr, out), stream)
    if r != 0:
        raise RuntimeError(f"matfun_gb300: kernel launch returned {r}")
    return tuple(out[:order + 1]) if order else out[0]


def smf(kind, A, alpha=None, order=0):
    """f(A) and its first and second derivatives for symmetric 3x3 matrices, as matrices A (..., 3, 3) or Voigt
    vectors A (..., 6) = (A11, A22, A33, A12, A13, A23); results in the same form:
        matrices:  F (..., 3, 3),  J (..., 3, 3, 3, 3),  H (..., 3, 3, 3, 3, 3, 3)
        Voigt:     F (..., 6),     J (..., 6, 6),        H (..., 6, 6, 6)
    order 0: F, 1: (F, J), 2: (F, J, H)."""
    _check(kind, alpha, order)
    A = _prep(A)
    lib = load()
    if tuple(A.shape[-2:]) == (3, 3):
        sh, shapes, fn = tuple(A.shape[:-2]), ((3, 3), (3, 3, 3, 3), (3, 3, 3, 3, 3, 3)), lib.smf_cuda_eval_matrix
    elif tuple(A.shape[-1:]) == (6,):
        sh, shapes, fn = tuple(A.shape[:-1]), ((6,), (6, 6), (6, 6, 6)), lib.smf_cuda_eval
    else:
        raise ValueError(f"expected matrices (..., 3, 3) or Voigt vectors (..., 6), got shape {tuple(A.shape)}")
    return _run(fn, kind, alpha, A, sh, shapes, order)


def gmf(kind, A, alpha=None, order=0):
    """f(A) and its first and second derivatives for general real 3x3 matrices A (..., 3, 3), principal branch:
    F (..., 3, 3), J (..., 3, 3, 3, 3), H (..., 3, 3, 3, 3, 3, 3); NaN for a matrix with a real eigenvalue <= 0
    (log, sqrt, pow)."""
    _check(kind, alpha, order)
    A = _prep(A)
    if tuple(A.shape[-2:]) != (3, 3):
        raise ValueError(f"expected matrices (..., 3, 3), got shape {tuple(A.shape)}")
    sh = tuple(A.shape[:-2])
    return _run(load().gmf_cuda_eval, kind, alpha, A, sh, ((3, 3), (3, 3, 3, 3), (3, 3, 3, 3, 3, 3)), order)

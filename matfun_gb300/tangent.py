"""The tangent of psi(A) = |f(A)|^2 / 2 for general 3x3 matrices on torch CUDA tensors (FP64), through gmf_cuda_tangent:
the value F = f(A), the gradient G = J^T F and the Hessian K = J^T J + F : H of psi, with J and H never formed
(81 + 9 + 9 doubles written per matrix instead of the 819 of F, J, H).  For f = log this is the tangent of the
Hencky-type potential |log A|^2 / 2 of a Newton method (the consumer-side contraction named in the reference's
theory.md:190):

    from matfun_gb300.tangent import gmf_tangent
    F, G, K = gmf_tangent("log", A)      # A (..., 3, 3) float64 CUDA -> F, G (..., 3, 3), K (..., 3, 3, 3, 3)
    psi = 0.5 * (F * F).sum((-2, -1))

K[..., c, d, e, f] = sum_ab (dF_ab/dA_cd dF_ab/dA_ef + F_ab d2F_ab/dA_cd dA_ef).  Same kinds and errors as gmf.
"""
import torch

from ._lib import KINDS, load


def gmf_tangent(kind, A, alpha=None, value=True, grad=True):
    """(F, G, K) of psi(A) = |f(A)|^2 / 2; F (value=False) and G (grad=False) may be skipped (None)"""
    if kind not in KINDS:
        raise ValueError(f"unknown function {kind!r}, expected one of {sorted(KINDS)}")
    if kind == "pow" and not (alpha is not None and alpha > 0):
        raise ValueError("pow needs an exponent alpha > 0")
    if A.shape[-2:] != (3, 3):
        raise ValueError(f"expected matrices (..., 3, 3), got shape {tuple(A.shape)}")
    if not A.is_cuda or A.dtype != torch.float64:
        raise TypeError("expected a float64 CUDA tensor")
    A = A.contiguous()
    sh = A.shape[:-2]
    n = A.numel() // 9
    F = torch.empty(sh + (3, 3), dtype=A.dtype, device=A.device) if value else None
    G = torch.empty(sh + (3, 3), dtype=A.dtype, device=A.device) if grad else None
    K = torch.empty(sh + (3, 3, 3, 3), dtype=A.dtype, device=A.device)
    p = lambda t: None if t is None else t.data_ptr()
    with torch.cuda.device(A.device):
        st = torch.cuda.current_stream().cuda_stream
        r = load().gmf_cuda_tangent(KINDS[kind], float(alpha or 0.0), n, A.data_ptr(), p(F), p(G), K.data_ptr(), st)
    if r != 0:
        raise RuntimeError(f"gmf_cuda_tangent returned {r}")
    return F, G, K

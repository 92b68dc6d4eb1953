"""Differentiable matrix functions on torch CUDA tensors, with the adjoint kernels of libmatfun_cuda:

    F = matfun_gb300.autograd.gmf("log", A)          # A (..., 3, 3) float64 CUDA, requires_grad
    L = (W * F).sum(); L.backward()                    # A.grad = J^T W       (gmf_cuda_adjoint, no J formed)
    g, = torch.autograd.grad(L, A, create_graph=True)
    (V * g).sum().backward()                           # W . H . V and J V    (no H formed)

The backward is itself a Function whose backward runs the Hessian contraction, so first and second derivatives
(double backward, Hessian-vector products) never materialise J or H; a third derivative raises.  float32 inputs run
the mixed-precision adjoint kernels (FP32 arrays and contractions).  smf treats A as
symmetric (derivatives of A -> f((A + A^T)/2), as the reference's smf_eval_matrix).  Functional forms: `adjoint`.
"""
import torch

from ._lib import KINDS, load


def _fn(fam, f32):
    lib = load()
    if f32:
        return lib.gmf_cuda_adjoint_f32 if fam == "gmf" else lib.smf_cuda_adjoint_f32
    return lib.gmf_cuda_adjoint if fam == "gmf" else lib.smf_cuda_adjoint


def adjoint(fam, kind, A, W=None, V=None, alpha=None, want=("F",)):
    """one launch of the adjoint kernel: returns a dict with the requested subset of
    F = f(A), Abar = J^T W, JV = J V, HWV = W . H . V (matrix layout, shapes of A).  float32 A runs the
    mixed-precision kernels (FP32 arrays); any other dtype runs in float64."""
    if fam not in ("smf", "gmf"):
        raise ValueError("fam must be 'smf' or 'gmf'")
    if kind not in KINDS:
        raise ValueError(f"unknown function {kind!r}, expected one of {sorted(KINDS)}")
    if kind == "pow" and not (alpha is not None and alpha > 0):
        raise ValueError("pow needs an exponent alpha > 0")
    if tuple(A.shape[-2:]) != (3, 3):
        raise ValueError(f"expected matrices (..., 3, 3), got shape {tuple(A.shape)}")
    if not A.is_cuda:
        raise TypeError("expected CUDA tensors")
    f32 = A.dtype == torch.float32
    dt = torch.float32 if f32 else torch.float64
    A = A.detach().to(dt).contiguous()
    W = None if W is None else W.detach().to(dt).expand_as(A).contiguous()
    V = None if V is None else V.detach().to(dt).expand_as(A).contiguous()
    out = {k: torch.empty_like(A) for k in want}
    p = lambda t: None if t is None else t.data_ptr()
    n = A.numel() // 9
    stream = torch.cuda.current_stream(A.device).cuda_stream
    with torch.cuda.device(A.device):
        r = _fn(fam, f32)(KINDS[kind], float(alpha or 0.0), n, p(A), p(W), p(V), p(out.get("F")),
                          p(out.get("Abar")), p(out.get("JV")), p(out.get("HWV")), stream)
    if r != 0:
        raise RuntimeError(f"matfun_gb300: adjoint kernel returned {r}")
    return out


class _Grad(torch.autograd.Function):
    """Abar = J(A)^T W; its own derivatives are W . H . V (w.r.t. A) and J V (w.r.t. W)"""

    @staticmethod
    def forward(ctx, A, W, fam, kind, alpha):
        ctx.save_for_backward(A, W)
        ctx.args = (fam, kind, alpha)
        return adjoint(fam, kind, A, W=W, alpha=alpha, want=("Abar",))["Abar"]

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, V):
        A, W = ctx.saved_tensors
        fam, kind, alpha = ctx.args
        r = adjoint(fam, kind, A, W=W, V=V, alpha=alpha, want=("HWV", "JV"))
        return r["HWV"], r["JV"], None, None, None


class _Fun(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, fam, kind, alpha):
        ctx.save_for_backward(A)
        ctx.args = (fam, kind, alpha)
        return adjoint(fam, kind, A, alpha=alpha, want=("F",))["F"]

    @staticmethod
    def backward(ctx, W):
        (A,) = ctx.saved_tensors
        fam, kind, alpha = ctx.args
        return _Grad.apply(A, W, fam, kind, alpha), None, None, None


def gmf(kind, A, alpha=None):
    """f(A) for general real 3x3 matrices A (..., 3, 3), differentiable twice through the adjoint kernels"""
    return _Fun.apply(A, "gmf", kind, alpha)


def smf(kind, A, alpha=None):
    """f(A) for symmetric 3x3 matrices A (..., 3, 3), differentiable twice through the adjoint kernels"""
    return _Fun.apply(A, "smf", kind, alpha)

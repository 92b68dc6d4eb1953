"""JAX front end with reverse-mode derivatives through the adjoint kernels (XLA FFI handlers of libmatfun_cuda on the
CUDA platform):

    import jax; jax.config.update("jax_enable_x64", True)
    from matfun_gb300 import jax as mj
    F = mj.gmf("log", A)                                    # A (..., 3, 3) float64 or float32 on a GPU
    L = lambda A: (W * mj.gmf("log", A)).sum()
    g = jax.grad(L)(A)                                      # J^T W (GmfAdjointCuda), no J formed
    hv = jax.grad(lambda A: (jax.grad(L)(A) * V).sum())(A)  # W . H . V, no H formed

f is a jax.custom_vjp whose backward (J^T W) is itself a custom_vjp whose backward runs the Hessian contraction
(W . H . V) and J V, so first and second reverse-mode derivatives never materialise J or H; a third derivative raises
(the contraction has no derivative rule), and forward mode (jvp, jacfwd, hessian) is not defined on custom_vjp.  smf
treats A as symmetric (the derivatives of A -> f((A + A^T) / 2)).  float32 arrays run the FP32 kernels.

gmf_tangent(kind, A) returns F, J^T F and J^T J + F : H of |f(A)|^2 / 2 in one custom call (GmfTangentCuda).

The values F, J, H themselves (order 0, 1, 2) are the reference's own matfun.jax over this library: it binds the
handlers SmfValueCuda ... GmfValueJacHessCuda that libmatfun_cuda exports (MATFUN_CUDA_LIB).
"""
import ctypes
import functools

import jax
import jax.numpy as jnp
import numpy as np

from ._lib import KINDS, library_path

OUT_F, OUT_ABAR, OUT_JV, OUT_HWV = 1, 2, 4, 8
_TARGETS = {("smf", False): ("matfun_gb300_smf_adjoint", "SmfAdjointCuda"),
            ("gmf", False): ("matfun_gb300_gmf_adjoint", "GmfAdjointCuda"),
            ("smf", True): ("matfun_gb300_smf_adjoint_f32", "SmfAdjointF32Cuda"),
            ("gmf", True): ("matfun_gb300_gmf_adjoint_f32", "GmfAdjointF32Cuda"),
            ("tangent", False): ("matfun_gb300_gmf_tangent", "GmfTangentCuda")}
_state = {"registered": False}


def _ffi():
    return jax.ffi if hasattr(jax, "ffi") else jax.extend.ffi


def _register():
    if _state["registered"]:
        return
    lib = ctypes.CDLL(library_path())
    for target, sym in _TARGETS.values():
        _ffi().register_ffi_target(target, _ffi().pycapsule(getattr(lib, sym)), platform="CUDA")
    _state["registered"] = True


def _norm(kind, alpha):
    if kind not in KINDS:
        raise ValueError(f"unknown function {kind!r}, expected one of {sorted(KINDS)}")
    if kind == "pow" and not (alpha is not None and float(alpha) > 0):
        raise ValueError("pow needs an exponent alpha > 0")
    return KINDS[kind], float(alpha or 0.0)


def adjoint(fam, kind, alpha, A, W=None, V=None, outputs=OUT_F):
    """one adjoint custom call: the outputs selected by the bit mask (F, J^T W, J V, W . H . V, in that order), each of
    the shape of A; W and V broadcast to A's shape"""
    _register()
    if A.shape[-2:] != (3, 3):
        raise ValueError(f"expected matrices (..., 3, 3), got shape {A.shape}")
    f32 = A.dtype == jnp.float32
    if not f32 and A.dtype != jnp.float64:
        raise TypeError("expected float32 or float64 arrays (float64 needs jax_enable_x64)")
    empty = jnp.zeros((0,), A.dtype)
    W = empty if W is None else jnp.broadcast_to(jnp.asarray(W, A.dtype), A.shape)
    V = empty if V is None else jnp.broadcast_to(jnp.asarray(V, A.dtype), A.shape)
    out = [jax.ShapeDtypeStruct(A.shape, A.dtype)] * bin(outputs).count("1")
    target = _TARGETS[(fam, f32)][0]
    try:
        call = _ffi().ffi_call(target, out, vmap_method="broadcast_all")
    except TypeError:  # jax releases before vmap_method
        call = _ffi().ffi_call(target, out, vectorized=True)
    return call(A, W, V, kind=np.int64(kind), alpha=np.float64(alpha), outputs=np.int64(outputs))


@functools.partial(jax.custom_vjp, nondiff_argnums=(0, 1, 2))
def _value(fam, kind, alpha, A):
    return adjoint(fam, kind, alpha, A, outputs=OUT_F)[0]


def _value_fwd(fam, kind, alpha, A):
    return _value(fam, kind, alpha, A), A


def _value_bwd(fam, kind, alpha, A, W):
    return (_gradient(fam, kind, alpha, A, W),)


_value.defvjp(_value_fwd, _value_bwd)


@functools.partial(jax.custom_vjp, nondiff_argnums=(0, 1, 2))
def _gradient(fam, kind, alpha, A, W):
    return adjoint(fam, kind, alpha, A, W=W, outputs=OUT_ABAR)[0]


def _gradient_fwd(fam, kind, alpha, A, W):
    return _gradient(fam, kind, alpha, A, W), (A, W)


def _gradient_bwd(fam, kind, alpha, res, V):
    A, W = res
    JV, HWV = adjoint(fam, kind, alpha, A, W=W, V=V, outputs=OUT_JV | OUT_HWV)
    return HWV, JV  # d<V, J^T W>/dA = W . H . V, d<V, J^T W>/dW = J V


_gradient.defvjp(_gradient_fwd, _gradient_bwd)


def gmf(kind, A, alpha=None):
    """f(A) for general real 3x3 matrices A (..., 3, 3), twice differentiable in reverse mode by the adjoint kernels"""
    k, a = _norm(kind, alpha)
    return _value("gmf", k, a, A)


def smf(kind, A, alpha=None):
    """f(A) for symmetric 3x3 matrices A (..., 3, 3), twice differentiable in reverse mode by the adjoint kernels"""
    k, a = _norm(kind, alpha)
    return _value("smf", k, a, A)


def gmf_tangent(kind, A, alpha=None):
    """(F, G, K) of psi(A) = |f(A)|^2 / 2 for general float64 matrices A (..., 3, 3): F = f(A), the gradient
    G = J^T F and the Hessian K = J^T J + F : H (..., 3, 3, 3, 3), one custom call (GmfTangentCuda) that never forms J
    or H; for f = log the tangent of the Hencky-type potential |log A|^2 / 2 (not differentiable itself)"""
    k, a = _norm(kind, alpha)
    _register()
    if A.shape[-2:] != (3, 3) or A.dtype != jnp.float64:
        raise TypeError("expected float64 matrices (..., 3, 3) (with jax_enable_x64)")
    out = [jax.ShapeDtypeStruct(A.shape, A.dtype), jax.ShapeDtypeStruct(A.shape, A.dtype),
           jax.ShapeDtypeStruct(A.shape[:-2] + (3, 3, 3, 3), A.dtype)]
    try:
        call = _ffi().ffi_call(_TARGETS[("tangent", False)][0], out, vmap_method="broadcast_all")
    except TypeError:  # jax releases before vmap_method
        call = _ffi().ffi_call(_TARGETS[("tangent", False)][0], out, vectorized=True)
    return tuple(call(A, kind=np.int64(k), alpha=np.float64(a), outputs=np.int64(7)))

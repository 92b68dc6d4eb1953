"""Adjoint kernels (gmf_cuda_adjoint / smf_cuda_adjoint) and the torch.autograd.Function built on them:
contractions J^T W, J V, W.H.V against the oracle's materialised J and H (<= 1e-12 relative), central finite
differences (h = 1e-6), torch's gradcheck / gradgradcheck, and NaN outside the domain."""
import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel

pytestmark = pytest.mark.gpu
CASES = [("gmf", "log", None), ("gmf", "pow", 0.3), ("gmf", "exp", None), ("gmf", "sqrt", None),
         ("smf", "log", None), ("smf", "pow", 0.3), ("smf", "exp", None), ("smf", "sqrt", None)]


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _inputs(fam, n, seed):
    from matfun_gb300 import workloads as w
    if fam == "gmf":
        A = w.c1_gmf_groups(n, seed=seed)
    else:
        A = w.c0_smf_spd(n, seed=seed, as_voigt=False)
    rng = np.random.default_rng(seed + 100)
    return A, rng.standard_normal((n, 3, 3)), rng.standard_normal((n, 3, 3))


@pytest.mark.parametrize("fam,kind,alpha", CASES)
def test_adjoint_matches_oracle_contractions(fam, kind, alpha):
    import torch

    from matfun_gb300.autograd import adjoint
    A, W, V = _inputs(fam, 2000, 3)
    r = adjoint(fam, kind, torch.from_numpy(A).cuda(), W=torch.from_numpy(W).cuda(), V=torch.from_numpy(V).cuda(),
                alpha=alpha, want=("F", "Abar", "JV", "HWV"))
    F, Jo, Ho = (ol.gmf if fam == "gmf" else ol.smf)(kind, A, alpha=alpha, order=2)
    Jo, Ho = Jo.reshape(-1, 3, 3, 3, 3), Ho.reshape(-1, 3, 3, 3, 3, 3, 3)
    ref = {"F": F,
           "Abar": np.einsum("nab,nabcd->ncd", W, Jo),
           "JV": np.einsum("nabcd,ncd->nab", Jo, V),
           "HWV": np.einsum("nab,nabcdef,ncd->nef", W, Ho, V)}
    for k in ref:
        got = r[k].cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(ref[k])), k
        ok = ~np.isnan(ref[k]).any(axis=(1, 2))
        assert maxrel(got[ok], ref[k][ok]) <= 1e-11, (k, maxrel(got[ok], ref[k][ok]))


@pytest.mark.parametrize("fam,kind,alpha", [("gmf", "log", None), ("gmf", "pow", 0.3), ("smf", "log", None)])
def test_autograd_against_central_differences(fam, kind, alpha):
    import torch

    import matfun_gb300
    from matfun_gb300 import autograd as ag
    A, W, V = _inputs(fam, 64, 5)
    A = A[np.isfinite(ol.gmf(kind, A, alpha=alpha)).all(axis=(1, 2))] if fam == "gmf" else A
    W, V = W[:len(A)], V[:len(A)]
    f = ag.gmf if fam == "gmf" else ag.smf
    tA = torch.from_numpy(A).cuda().requires_grad_(True)
    tW, tV = torch.from_numpy(W).cuda(), torch.from_numpy(V).cuda()
    L = (tW * f(kind, tA, alpha=alpha)).sum()
    (g,) = torch.autograd.grad(L, tA, create_graph=True)
    (hv,) = torch.autograd.grad((tV * g).sum(), tA)
    ev = (lambda X: matfun_gb300.gmf(kind, X, alpha=alpha)) if fam == "gmf" else (lambda X: matfun_gb300.smf(kind, X, alpha=alpha))
    h = 1e-6
    Vs = tV if fam == "gmf" else 0.5 * (tV + tV.transpose(1, 2))
    # directional derivative of L along V, and of the gradient along V
    dL = ((tW * ev(tA.detach() + h * Vs)).sum() - (tW * ev(tA.detach() - h * Vs)).sum()) / (2 * h)
    gv = float((g.detach() * Vs).sum())
    assert abs(float(dL) - gv) <= 1e-6 * max(1.0, abs(float(dL)))
    gp = ag.adjoint(fam, kind, tA.detach() + h * Vs, W=tW, alpha=alpha, want=("Abar",))["Abar"]
    gm = ag.adjoint(fam, kind, tA.detach() - h * Vs, W=tW, alpha=alpha, want=("Abar",))["Abar"]
    fd = (gp - gm) / (2 * h)
    hvs = hv if fam == "gmf" else 0.5 * (hv + hv.transpose(1, 2))
    fds = fd if fam == "gmf" else 0.5 * (fd + fd.transpose(1, 2))
    assert float((hvs - fds).abs().max()) <= 1e-5 * max(1.0, float(fds.abs().max()))


def test_gradcheck_and_gradgradcheck():
    import torch

    from matfun_gb300 import autograd as ag
    rng = np.random.default_rng(0)
    A = torch.from_numpy(np.eye(3) + 0.3 * rng.standard_normal((4, 3, 3))).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda X: ag.gmf("log", X), (A,), eps=1e-6, atol=1e-6)
    assert torch.autograd.gradgradcheck(lambda X: ag.gmf("log", X), (A,), eps=1e-6, atol=1e-5)
    S = torch.from_numpy(np.eye(3) * 2 + 0.1 * rng.standard_normal((4, 3, 3))).cuda()
    S = (0.5 * (S + S.transpose(1, 2))).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda X: ag.smf("sqrt", 0.5 * (X + X.transpose(1, 2))), (S,), eps=1e-6, atol=1e-6)


def test_third_derivative_refused_and_domain_nan():
    import torch

    from matfun_gb300 import autograd as ag
    A = torch.diag(torch.tensor([-1.0, 2.0, 3.0], dtype=torch.float64)).cuda()[None].requires_grad_(True)
    F = ag.gmf("log", A)
    assert bool(torch.isnan(F).all())
    B = (torch.eye(3, dtype=torch.float64).cuda() * 2)[None].requires_grad_(True)
    (g,) = torch.autograd.grad(ag.gmf("log", B).sum(), B, create_graph=True)
    (h,) = torch.autograd.grad(g.sum(), B, create_graph=True)
    with pytest.raises(RuntimeError):
        torch.autograd.grad(h.sum(), B)


@pytest.mark.parametrize("fam,kind,alpha", CASES)
def test_adjoint_f32_against_fp64(fam, kind, alpha):
    """the mixed-precision adjoints (smf_cuda_adjoint_f32 / gmf_cuda_adjoint_f32) against the FP64 adjoints on the
    same FP32 values: max |x - ref| / max |ref| per output <= 1e-6, identical NaN positions; smf on the C2 workload
    (condition numbers to 1e6, gaps to 1e-12), gmf on the C1 groups"""
    import torch

    from matfun_gb300 import workloads as w
    from matfun_gb300.autograd import adjoint
    n = 16000
    A = (w.c1_gmf_groups(n, seed=11) if fam == "gmf" else w.c2_smf_spd(n, seed=11, as_voigt=False)).astype(np.float32)
    rng = np.random.default_rng(12)
    W = rng.standard_normal((n, 3, 3)).astype(np.float32)
    V = rng.standard_normal((n, 3, 3)).astype(np.float32)
    want = ("F", "Abar", "JV", "HWV")
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    r32 = adjoint(fam, kind, t(A), W=t(W), V=t(V), alpha=alpha, want=want)
    r64 = adjoint(fam, kind, t(A).double(), W=t(W).double(), V=t(V).double(), alpha=alpha, want=want)
    errs = {}
    for k in want:
        assert r32[k].dtype == torch.float32 and r64[k].dtype == torch.float64
        got, ref = r32[k].double().cpu().numpy(), r64[k].cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(ref)), k
        errs[k] = maxrel(got, ref)
    print(f"adjoint f32 {fam} {kind} {alpha}: " + " ".join(f"{k} {e:.2e}" for k, e in errs.items()))
    assert max(errs.values()) <= 1e-6, errs


def test_autograd_f32_gradient_and_hvp():
    """float32 tensors run the FP32 adjoint kernels through autograd: gradient and Hessian-vector product close to the
    float64 ones"""
    import torch

    from matfun_gb300 import autograd as ag
    from matfun_gb300 import workloads as w
    A = torch.from_numpy(w.c0_smf_spd(512, seed=4, as_voigt=False).astype(np.float32)).cuda()
    Wd = torch.randn(512, 3, 3, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    Vd = torch.randn(512, 3, 3, device="cuda", generator=torch.Generator("cuda").manual_seed(2))
    out = {}
    for dt in (torch.float32, torch.float64):
        X = A.to(dt).requires_grad_(True)
        L = (Wd.to(dt) * ag.smf("log", X)).sum()
        g, = torch.autograd.grad(L, X, create_graph=True)
        hv, = torch.autograd.grad((g * Vd.to(dt)).sum(), X)
        out[dt] = (g.detach(), hv)
        assert g.dtype == dt and hv.dtype == dt
    for a, b in zip(out[torch.float32], out[torch.float64]):
        assert float((a.double() - b).abs().max() / b.abs().max()) <= 1e-6

"""The tangent of psi(A) = |f(A)|^2 / 2 (gmf_cuda_tangent: F, G = J^T F, K = J^T J + F : H without forming J or H)
against the same contractions of the oracle's F, J, H.  Tolerance: max |x - ref| / max |ref| <= 1e-12 per call and
output (the FP64 path's parity bound); NaN exactly where the oracle has NaN; K symmetric."""
import ctypes

import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel

pytestmark = pytest.mark.gpu
TOL = 1e-12
KINDS = [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3"), (2, 1.7, "pow 1.7")]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def tangent_gpu(kind, alpha, X, value=True, grad=True):
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    n = len(X)
    dX = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).cuda()
    F = torch.full((n, 9), -7.0, dtype=torch.float64, device="cuda") if value else None
    G = torch.full((n, 9), -7.0, dtype=torch.float64, device="cuda") if grad else None
    K = torch.full((n, 81), -7.0, dtype=torch.float64, device="cuda")
    p = lambda t: None if t is None else t.data_ptr()
    r = lib.gmf_cuda_tangent(kind, alpha, n, dX.data_ptr(), p(F), p(G), K.data_ptr(),
                             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert r == 0
    return [None if t is None else t.cpu().numpy() for t in (F, G, K)]


def tangent_oracle(kind, alpha, X):
    """F, G = J^T F, K = J^T J + F : H from the oracle's F, J (9 x 9: output x input) and H (9 x 9 x 9)"""
    r, F, J, H = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X, 2, 9)
    assert r == 0
    n = len(X)
    Jm, Hm = J.reshape(n, 9, 9), H.reshape(n, 9, 9, 9)
    G = np.einsum("nm,nmc->nc", F, Jm)
    K = np.einsum("nmc,nme->nce", Jm, Jm) + np.einsum("nm,nmce->nce", F, Hm)
    return F, G, K.reshape(n, 81)


def _cmp(kind, alpha, X, name):
    got = tangent_gpu(kind, alpha, X)
    ref = tangent_oracle(kind, alpha, X)
    errs = []
    for g, o, nm in zip(got, ref, "FGK"):
        assert np.array_equal(np.isnan(g), np.isnan(o)), f"{name} {nm}: NaN positions differ"
        errs.append(maxrel(g, o))
    K = got[2].reshape(-1, 9, 9)
    ok = ~np.isnan(K).any(axis=(1, 2))
    sym = np.abs(K[ok] - K[ok].transpose(0, 2, 1)).max(initial=0.0) / max(np.abs(K[ok]).max(initial=0.0), 1e-300)
    print(f"tangent {name} n={len(X)}: max rel F {errs[0]:.1e} G {errs[1]:.1e} K {errs[2]:.1e}, asym {sym:.1e}")
    assert max(errs) <= TOL, (name, errs)
    assert sym <= TOL
    return got, ref


@pytest.mark.parametrize("kind,alpha,name", KINDS)
def test_tangent_c1_groups(kind, alpha, name):
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(4 * 1500, seed=21).reshape(-1, 9)
    X[7] = [-1, 0, 0, 0, 2, 0, 0, 0, 3]  # eigenvalue -1: NaN for log, sqrt, pow
    _cmp(kind, alpha, X, name)


@pytest.mark.parametrize("kind,alpha,name", KINDS[1:3])
def test_tangent_ordered_launch(kind, alpha, name):
    """n >= 2^15: the batch-ordered launch with its plain tail (whose rows of K held the scratch).  F equals the
    order-2 evaluation's F bit for bit (the same ordered launch), and G, K equal the contractions of that
    evaluation's own J and H to 1e-12.  (This batch holds a rotation x stretch matrix near the branch cut with
    entries of log A near 1e3, where every FP64 evaluation differs from the oracle by ~1e-10 of the batch's largest
    value: the conditioning of log there, not the contraction.)"""
    from tests.gpu_util import gpu_call
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(40000, seed=22).reshape(-1, 9)
    F, G, K = tangent_gpu(kind, alpha, X)
    assert not (K == -7.0).any()  # every row written, the scratch rows included
    r, Fe, Je, He = gpu_call("gmf_eval", kind, alpha, X, 2, 9)
    assert r == 0
    assert np.array_equal(F, Fe, equal_nan=True)
    n = len(X)
    Jm, Hm = Je.reshape(n, 9, 9), He.reshape(n, 9, 9, 9)
    Gr = np.einsum("nm,nmc->nc", Fe, Jm)
    Kr = (np.einsum("nmc,nme->nce", Jm, Jm) + np.einsum("nm,nmce->nce", Fe, Hm)).reshape(n, 81)
    for a, b in ((G, Gr), (K, Kr)):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert maxrel(a, b) <= TOL


def _term_scale(F, J, H):
    """per matrix: the largest sum of the magnitudes of the terms that make up an entry of G and of K (the scale of
    the rounding of any correct evaluation of the contractions)"""
    n = len(F)
    aF, aJ, aH = np.abs(F), np.abs(J.reshape(n, 9, 9)), np.abs(H.reshape(n, 9, 9, 9))
    sG = np.einsum("nm,nmc->nc", aF, aJ).max(axis=1)
    sK = (np.einsum("nmc,nme->nce", aJ, aJ) + np.einsum("nm,nmce->nce", aF, aH)).reshape(n, 81).max(axis=1)
    return sG, sK


def test_tangent_golden_inputs():
    """the reference's golden gmf inputs: G, K against the contractions of this library's own order-2 evaluation
    (1e-12 of the terms' magnitude per matrix), and against those of the oracle's F, J, H within 10x the case's
    golden tolerance of the same scale (the ill-conditioned cases have |K| far below |J|^2 + |F||H|)"""
    import os

    from tests.gpu_util import gpu_call
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cases_gmf.npz"))
    for kind in np.unique(g["kind"]):
        for alpha in np.unique(g["alpha"][g["kind"] == kind]):
            sel = np.where((g["kind"] == kind) & (g["alpha"] == alpha))[0]
            X = g["x"][sel]
            F, G, K = tangent_gpu(int(kind), float(alpha), X)
            r, Fe, Je, He = gpu_call("gmf_eval", int(kind), float(alpha), X, 2, 9)
            assert r == 0 and np.array_equal(F, Fe, equal_nan=True)
            n = len(X)
            sG, sK = _term_scale(Fe, Je, He)
            for ref, bound in ((tangent_oracle(int(kind), float(alpha), X), 10 * np.maximum(g["tol"][sel], TOL)),
                               ((Fe, np.einsum("nm,nmc->nc", Fe, Je.reshape(n, 9, 9)),
                                 (np.einsum("nmc,nme->nce", Je.reshape(n, 9, 9), Je.reshape(n, 9, 9)) +
                                  np.einsum("nm,nmce->nce", Fe, He.reshape(n, 9, 9, 9))).reshape(n, 81)),
                                np.full(n, TOL))):
                for a, b, sc in ((G, ref[1], sG), (K, ref[2], sK)):
                    assert np.array_equal(np.isnan(a), np.isnan(b))
                    d = np.where(np.isnan(a) & np.isnan(b), 0.0, np.abs(a - b)).max(axis=1)
                    ok = ~np.isnan(sc)
                    assert np.all(d[ok] <= bound[ok] * sc[ok]), (int(kind), float(alpha), np.max(d[ok] / sc[ok]))


def test_tangent_optional_outputs_and_errors():
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(400, seed=23).reshape(-1, 9)
    F, G, K = tangent_gpu(1, 0.0, X)
    F2, G2, K2 = tangent_gpu(1, 0.0, X, value=False, grad=False)
    assert F2 is None and G2 is None and np.array_equal(K, K2, equal_nan=True)
    lib = matfun_gb300.load()
    dX = torch.from_numpy(X).cuda()
    dK = torch.empty((len(X), 81), dtype=torch.float64, device="cuda")
    assert lib.gmf_cuda_tangent(7, 0.0, len(X), dX.data_ptr(), None, None, dK.data_ptr(), None) == -1
    assert lib.gmf_cuda_tangent(2, 0.0, len(X), dX.data_ptr(), None, None, dK.data_ptr(), None) == -1
    assert lib.gmf_cuda_tangent(1, 0.0, len(X), dX.data_ptr(), None, None, None, None) == -1
    assert lib.gmf_cuda_tangent(1, 0.0, -1, dX.data_ptr(), None, None, dK.data_ptr(), None) == -1
    assert lib.gmf_cuda_tangent(1, 0.0, 0, None, None, None, None, None) == 0


def test_tangent_torch_front_end():
    import torch

    from matfun_gb300.tangent import gmf_tangent
    from matfun_gb300 import workloads as w
    A = torch.from_numpy(w.c1_gmf_groups(64, seed=24)).cuda().reshape(4, 16, 3, 3)
    F, G, K = gmf_tangent("log", A)
    assert F.shape == (4, 16, 3, 3) and G.shape == (4, 16, 3, 3) and K.shape == (4, 16, 3, 3, 3, 3)
    ref = tangent_oracle(1, 0.0, A.reshape(-1, 9).cpu().numpy())
    assert maxrel(K.reshape(-1, 81).cpu().numpy(), ref[2]) <= TOL
    # the Newton step of psi: K (as 9 x 9) against finite differences of G = grad psi
    h = 1e-6
    A0 = A.reshape(-1, 3, 3)[:8]
    _, G0, K0 = gmf_tangent("log", A0)
    for q in range(9):
        E = torch.zeros(9, dtype=torch.float64, device="cuda")
        E[q] = h
        _, Gp, _ = gmf_tangent("log", A0 + E.reshape(3, 3))
        _, Gm, _ = gmf_tangent("log", A0 - E.reshape(3, 3))
        fd = ((Gp - Gm) / (2 * h)).reshape(-1, 9)
        col = K0.reshape(-1, 9, 9)[:, :, q]
        assert (fd - col).abs().max() <= 1e-6 * col.abs().max()
    with pytest.raises(ValueError):
        gmf_tangent("pow", A)
    with pytest.raises(TypeError):
        gmf_tangent("log", A.float())

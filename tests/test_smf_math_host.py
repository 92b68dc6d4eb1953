"""The per-matrix math of the symmetric family, held against the oracle on the CPU.

The eigensystem, f of the eigenvalues and the first / second divided differences that the smf kernels evaluate per
thread (FP32 mixed form: matfun_gb300/csrc/smf_mixed_math.cuh; FP64 form: smf_device.cuh) are compiled for the host
from the same headers with g++ (tests/host_math/smf_math_host.cc; host_intrinsics.h supplies the six CUDA intrinsics
they use as exact host functions).  F, J and H are assembled from V, f(lambda), D and D2 in NumPy by the spectral
(Daleckii-Krein) formulas and compared with the oracle's smf_eval_matrix:

    F            = V diag(f) V^T
    J[ij, kl]    = sum_ab V_ia V_jb D_ab Xt_kl,ab,                         Xt_kl = V^T (E_kl + E_lk) / 2 V
    H[ij, kl, pq] = sum_abc V_ia V_jb D2_acb (Xt_kl,ac Xt_pq,cb + Xt_pq,ac Xt_kl,cb)

This checks the math without a GPU (the device's own math library and the tile's FP32 assembly are checked by the
GPU tests).  Bounds: 1e-6 for the FP32 form (max |x - ref| / max |ref| per array, as tests/test_mixed_gpu.py), 1e-12
for the FP64 form (as tests/test_parity_gpu.py)."""
import ctypes
import os

import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import build_host_math, maxrel, near_degenerate_f32

HERE = os.path.dirname(os.path.abspath(__file__))
KINDS = [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3"), (2, 0.7, "pow 0.7")]
P = ctypes.c_void_p


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = build_host_math("smf_math_host.cc", tmp_path_factory.mktemp("host_math"), "-O2")
    if out is None:
        pytest.skip("g++ or the CUDA headers are missing")
    L = ctypes.CDLL(out)
    L.smf_math_f32.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int64] + [P] * 6
    L.smf_math_f64.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [P] * 6
    L.smf_math_f32.restype = L.smf_math_f64.restype = ctypes.c_int
    return L


def spectra(L, kind, alpha, X, f32, mat=True):
    n = len(X)
    dt = np.float32 if f32 else np.float64
    X = np.ascontiguousarray(X, dtype=dt)
    lam, fl = np.empty((n, 3), dt), np.empty((n, 3), dt)
    V, D, D2 = np.empty((n, 3, 3), dt), np.empty((n, 3, 3), dt), np.empty((n, 3, 3, 3), dt)
    outs = [a.ctypes.data for a in (lam, fl, V, D, D2)]
    if f32:
        assert L.smf_math_f32(kind, alpha, int(mat), n, X.ctypes.data, *outs) == 0
    else:
        assert L.smf_math_f64(kind, alpha, n, X.ctypes.data, *outs) == 0
    return [a.astype(np.float64) for a in (lam, fl, V, D, D2)]


def assemble(fl, V, D, D2):
    """F (n, 9), J (n, 81), H (n, 729) in the matrix layout of smf_eval_matrix"""
    n = len(V)
    F = np.einsum("nia,na,nja->nij", V, fl, V)
    Xt = 0.5 * (np.einsum("nka,nlb->nklab", V, V) + np.einsum("nla,nkb->nklab", V, V)).reshape(n, 9, 3, 3)
    J = np.einsum("nia,njb,nab,nKab->nijK", V, V, D, Xt, optimize=True)
    M = np.einsum("nacb,nKac,nPcb->nKPab", D2, Xt, Xt, optimize=True)
    H = np.einsum("nia,njb,nKPab->nijKP", V, V, M + M.transpose(0, 2, 1, 3, 4), optimize=True)
    return F.reshape(n, 9), J.reshape(n, 81), H.reshape(n, 729)


def voigt(A):
    return np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], axis=1)


def inputs():
    from matfun_gb300 import workloads as w
    return {
        "C2": w.c2_smf_spd(2000, seed=31, as_voigt=False),
        "C0": w.c0_smf_spd(2000, seed=32, as_voigt=False),
        "near-isotropic": near_degenerate_f32().astype(np.float64),
    }


@pytest.mark.parametrize("kind,alpha,name", KINDS)
def test_fp32_math_against_oracle(lib, kind, alpha, name):
    for case, A in inputs().items():
        A32 = A.astype(np.float32)
        ref = ol.call(ol.oracle(), "smf_eval_matrix", kind, alpha, A32.astype(np.float64).reshape(-1, 9), 2, 9)[1:]
        for layout, X in (("matrix", A32.reshape(-1, 9)), ("Voigt", voigt(A32))):
            _, fl, V, D, D2 = spectra(lib, kind, alpha, X, True, mat=layout == "matrix")
            errs = [maxrel(g, r) for g, r in zip(assemble(fl, V, D, D2), ref)]
            print(f"FP32 smf math, {name}, {case}, {layout}: max rel F J H {['%.1e' % e for e in errs]}")
            assert max(errs) <= 1e-6, (case, layout, errs)


def test_fp32_eigenvectors_orthonormal(lib):
    """every FP32 eigenvector matrix orthonormal to FP32 rounding, row by row (a size-independent property): near-
    degenerate pairs whose Jacobi block squares below FP32's normal range left V^T V 1e-5 .. 1.5e-2 from I before
    the block was scaled by a power of two"""
    from matfun_gb300 import workloads as w
    X = np.concatenate([A.astype(np.float32).reshape(-1, 9) for A in inputs().values()] +
                       [w.c0_smf_spd(50000, seed=6, as_voigt=False).astype(np.float32).reshape(-1, 9)])
    _, _, V, _, _ = spectra(lib, 1, 0.0, X, True)
    err = np.abs(np.einsum("nia,nib->nab", V, V) - np.eye(3)).reshape(len(X), -1).max(1)
    print(f"FP32 eigenvectors: max |V^T V - I| {err.max():.1e} over {len(X)} matrices")
    assert err.max() <= 2e-7, (int(err.argmax()), float(err.max()))


@pytest.mark.parametrize("kind,alpha,name", KINDS)
def test_fp64_math_against_oracle(lib, kind, alpha, name):
    for case, A in inputs().items():
        ref = ol.call(ol.oracle(), "smf_eval_matrix", kind, alpha, A.reshape(-1, 9), 2, 9)[1:]
        _, fl, V, D, D2 = spectra(lib, kind, alpha, voigt(A), False)
        errs = [maxrel(g, r) for g, r in zip(assemble(fl, V, D, D2), ref)]
        print(f"FP64 smf math, {name}, {case}: max rel F J H {['%.1e' % e for e in errs]}")
        assert max(errs) <= 1e-12, (case, errs)


VPAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def to_voigt(F, J, H):
    """matrix-layout F, J, H of the symmetric part -> the Voigt layout of smf_eval: a Voigt direction of an
    off-diagonal pair moves A_kl and A_lk together, so its derivative is the sum over both entries"""
    n = len(F)
    F9, J9, H9 = F.reshape(n, 3, 3), J.reshape(n, 3, 3, 3, 3), H.reshape(n, 3, 3, 3, 3, 3, 3)
    dirs = [[(k, l)] if k == l else [(k, l), (l, k)] for k, l in VPAIRS]
    Fv = np.stack([F9[:, i, j] for i, j in VPAIRS], 1)
    Jv = np.stack([np.stack([sum(J9[:, i, j, k, l] for k, l in dirs[p]) for p in range(6)], 1)
                   for i, j in VPAIRS], 1)
    Hv = np.stack([np.stack([np.stack([sum(H9[:, i, j, k, l, r, s] for k, l in dirs[p] for r, s in dirs[q])
                                       for q in range(6)], 1) for p in range(6)], 1) for i, j in VPAIRS], 1)
    return Fv, Jv.reshape(n, 36), Hv.reshape(n, 216)


@pytest.mark.parametrize("fixture,f32", [("cases_smf.npz", False), ("cases_smf_f32.npz", True)])
def test_golden_cases(lib, fixture, f32):
    """every golden smf case of the reference within its own tolerance (FP64 math), and the FP32-rounded golden
    inputs within the FP32 path's stated tolerance (FP32 math)"""
    g = np.load(os.path.join(HERE, "golden", fixture))
    worst = 0.0
    for kind in np.unique(g["kind"]):
        for alpha in np.unique(g["alpha"][g["kind"] == kind]):
            sel = np.where((g["kind"] == kind) & (g["alpha"] == alpha))[0]
            _, fl, V, D, D2 = spectra(lib, int(kind), float(alpha), g["x"][sel], f32, mat=False)
            got = to_voigt(*assemble(fl, V, D, D2))
            for row, i in enumerate(sel):
                for arr, name in zip(got, "FJH"):
                    e = maxrel(arr[row], g[name][i])
                    worst = max(worst, e / g["tol"][i])
                    assert e <= g["tol"][i], f"case {i} (kind {kind}, alpha {alpha}) {name}: {e:.2e}"
    print(f"{fixture}, {'FP32' if f32 else 'FP64'} math: worst {worst:.2f} of the case tolerance")


def stress_sets_spd(n, seed=11):
    """symmetric positive definite matrices the workloads do not stress: scaled by 2^-100 .. 2^100, pairs with relative
    gaps 1e-4 .. 1e-30, triples spread by 1e-6 .. 1e-20, condition number 1e6 (random rotations)"""
    rng = np.random.default_rng(seed)

    def spd(lam):
        Q, _ = np.linalg.qr(rng.standard_normal((len(lam), 3, 3)))
        return np.einsum("nia,na,nja->nij", Q, lam, Q)

    base = np.exp(rng.uniform(-1, 1, (n, 3)))
    sets = {f"scale 2^{k}": spd(base) * 2.0 ** k for k in (-100, -60, -20, 20, 60, 100)}
    for g in (1e-4, 1e-8, 1e-12, 1e-16, 1e-20, 1e-30):
        c, d = np.exp(rng.uniform(-1, 1, n)), np.exp(rng.uniform(-1, 1, n))
        sets[f"pair gap {g:.0e}"] = spd(np.stack([c, c * (1 + g), d], 1))
    for g in (1e-6, 1e-10, 1e-20):
        c = np.exp(rng.uniform(-1, 1, n))
        sets[f"triple spread {g:.0e}"] = spd(np.stack([c, c * (1 + g), c * (1 + 2 * g)], 1))
    sets["cond 1e6"] = spd(np.stack([np.ones(n), np.exp(rng.uniform(0, np.log(1e6), n)), 1e6 * np.ones(n)], 1))
    return sets


@pytest.mark.parametrize("kind,alpha,name", KINDS)
def test_fp64_math_stress(lib, kind, alpha, name):
    """the FP64 math on the stress sets within 1e-12 of the oracle (exp: only where exp of the spectrum is finite)"""
    for sname, A in stress_sets_spd(200).items():
        if kind == 0 and np.abs(A).max() > 80:  # exp overflows there in any precision
            continue
        A = 0.5 * (A + A.transpose(0, 2, 1))
        ref = ol.call(ol.oracle(), "smf_eval_matrix", kind, alpha, A.reshape(-1, 9), 2, 9)[1:]
        _, fl, V, D, D2 = spectra(lib, kind, alpha, voigt(A), False)
        errs = [maxrel(g, r) for g, r in zip(assemble(fl, V, D, D2), ref)]
        assert max(errs) <= 1e-12, (sname, errs)


def test_fp32_log_jacobian_free_of_scale(lib):
    """log J of the FP32 math per matrix (max error / max |J| of that matrix) within 6e-7 at |A| from 2^-60 to 2^60:
    the far-pair divided difference is log1p((b - a) / a) / (b - a) (the difference of two logs it replaced lost
    one ulp of log |A|: 1.3e-6 at 2^60)"""
    from tests.helpers import maxrel_rows
    for sname, A in stress_sets_spd(200).items():
        if not sname.startswith("scale") or abs(int(sname.split("^")[1])) > 60:
            continue
        A32 = (0.5 * (A + A.transpose(0, 2, 1))).astype(np.float32)
        ref = ol.call(ol.oracle(), "smf_eval_matrix", 1, 0.0, A32.astype(np.float64).reshape(-1, 9), 1, 9)
        _, fl, V, D, D2 = spectra(lib, 1, 0.0, A32.reshape(-1, 9), True)
        F, J, _ = assemble(fl, V, D, D2)
        e = maxrel_rows(J, ref[2]).max()
        assert e <= 6e-7, (sname, e)

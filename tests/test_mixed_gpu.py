"""The mixed-precision paths (smf_cuda_eval_f32 / smf_cuda_eval_matrix_f32 / gmf_cuda_eval_f32: FP32 storage, FP32
bulk arithmetic, FP64 only where FP32 would lose the result) against the FP64 oracle evaluated on the same FP32
input values.  Two error measures, F, J, H separately: per call, max |x - ref| / max |ref| over the output array;
and per matrix, the same within each matrix's row, over the matrices whose outputs fit FP32's range.  The bound is
1e-6 (the target of the mixed form) for both, except where a kind's own conditioning is stated below."""
import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel, maxrel_rows_fp32, near_degenerate_f32, random_general

pytestmark = pytest.mark.gpu
KINDS = [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3"), (2, 0.7, "pow 0.7")]
TOL = 1e-6
# per matrix, smf H on C2 (condition numbers up to 1e6): the FP32 eigenvector of a small separated eigenvalue is
# within about 2.5 ulp, and H carries six factors of it (measured on the host build, 100 000 C2 matrices: log and
# sqrt 1.2e-6, pow 0.7 2.3e-6; exp 5.8e-7)
SMF_PM_H = 2.5e-6


def run_f32(mat, kind, alpha, X32, order):
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    nf = 9 if mat else 6
    n = len(X32)
    dX = torch.from_numpy(np.ascontiguousarray(X32)).cuda()
    out = [torch.full((n, nf ** (k + 1)), 7.0, dtype=torch.float32, device="cuda") for k in range(order + 1)]
    out += [None] * (2 - order)
    p = lambda t: None if t is None else t.data_ptr()
    fn = lib.smf_cuda_eval_matrix_f32 if mat else lib.smf_cuda_eval_f32
    r = fn(kind, alpha, n, dX.data_ptr(), *map(p, out), None)
    torch.cuda.synchronize()
    assert r == 0
    return [t.cpu().numpy().astype(np.float64) for t in out[:order + 1]]


def errors(mat, kind, alpha, X32, order):
    got = run_f32(mat, kind, alpha, X32, order)
    fam = "smf_eval_matrix" if mat else "smf_eval"
    ref = ol.call(ol.oracle(), fam, kind, alpha, X32.astype(np.float64).reshape(len(X32), -1), order, 9 if mat else 6)
    return [maxrel(g, r) for g, r in zip(got, ref[1:order + 2])], got, ref


def per_matrix(got, ref):
    """the largest per-matrix error of each output (F, J, H)"""
    return [float(np.max(maxrel_rows_fp32(g, r), initial=0.0)) for g, r in zip(got, ref)]


@pytest.mark.parametrize("kind,alpha,name", KINDS)
@pytest.mark.parametrize("order", [0, 1, 2])
def test_smf_mixed_c2_voigt(kind, alpha, name, order):
    from matfun_gb300 import workloads as w
    X = w.c2_smf_spd(20000, seed=2 + order)
    errs, got, ref = errors(False, kind, alpha, X, order)
    pm = per_matrix(got, ref[1:])
    print(f"mixed smf Voigt {name} order {order}: per call / per matrix " +
          " ".join(f"{n} {e:.2e} / {p:.2e}" for n, e, p in zip("FJH", errs, pm)))
    for g, r in zip(got, ref[1:]):
        assert np.array_equal(np.isnan(g), np.isnan(r))
    assert max(errs) <= TOL
    assert max(pm[:2]) <= TOL
    assert order < 2 or pm[2] <= SMF_PM_H


@pytest.mark.parametrize("kind,alpha,name", KINDS[:3])
def test_smf_mixed_matrix_layout(kind, alpha, name):
    from matfun_gb300 import workloads as w
    A = w.c2_smf_spd(5000, seed=7, as_voigt=False)
    A[11, 0, 2] += 1.0  # not symmetric: NaN results
    errs, got, ref = errors(True, kind, alpha, A.reshape(-1, 9), 2)
    assert np.isnan(got[0][11]).all()
    assert max(errs) <= TOL


def test_smf_mixed_c0_and_golden_inputs():
    """the C0 workload (repeated eigenvalues) and the golden inputs, rounded to FP32"""
    import os

    from matfun_gb300 import workloads as w
    X = w.c0_smf_spd(20000, seed=0).astype(np.float32)
    errs, _, _ = errors(False, 1, 0.0, X, 2)
    assert max(errs) <= TOL
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cases_smf.npz"))
    sel = (g["kind"] == 1) & (np.abs(g["x"]).max(axis=1) < 1e30) & (np.abs(g["x"]).max(axis=1) > 1e-30)
    errs, _, _ = errors(False, 1, 0.0, g["x"][sel].astype(np.float32), 2)
    assert max(errs) <= 1e-5


@pytest.mark.parametrize("kind,alpha,name", KINDS)
def test_smf_mixed_near_isotropic(kind, alpha, name):
    A = near_degenerate_f32()
    errs, got, ref = errors(True, kind, alpha, A.reshape(-1, 9), 2)
    row = [maxrel(g[:1], r[:1]) for g, r in zip(got, ref[1:])]
    print(f"mixed smf near-isotropic {name}: max rel F J H {errs}; C0 row 29913 alone {row}")
    assert max(errs) <= TOL and max(row) <= TOL


def test_smf_mixed_adjoint_near_isotropic():
    """the FP32 VJP against the FP64 one on the same FP32 inputs (log: on a multiple of I, Abar = sym(W) / c)"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    A32 = torch.from_numpy(near_degenerate_f32()).cuda()
    n = A32.shape[0]
    W32 = torch.from_numpy(np.random.default_rng(5).standard_normal((n, 3, 3)).astype(np.float32)).cuda()
    Ab32 = torch.empty_like(A32)
    A64, W64 = A32.double(), W32.double()
    Ab64 = torch.empty_like(A64)
    assert lib.smf_cuda_adjoint_f32(1, 0.0, n, A32.data_ptr(), W32.data_ptr(), None, None, Ab32.data_ptr(),
                                    None, None, None) == 0
    assert lib.smf_cuda_adjoint(1, 0.0, n, A64.data_ptr(), W64.data_ptr(), None, None, Ab64.data_ptr(),
                                None, None, None) == 0
    torch.cuda.synchronize()
    err = maxrel(Ab32.double().cpu().numpy(), Ab64.cpu().numpy())
    print(f"mixed smf adjoint near-isotropic log: max rel Abar {err:.2e}")
    assert err <= TOL


# ---- general family (gmf_cuda_eval_f32): FP64 spectral analysis and series, FP32 storage and J / H assembly
GMF_KINDS = [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3")]
GMF_TOL = 1e-6


def gmf_errors(kind, alpha, X32, order):
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    n = len(X32)
    dX = torch.from_numpy(np.ascontiguousarray(X32.reshape(n, 9))).cuda()
    out = [torch.full((n, 9 ** (k + 1)), 7.0, dtype=torch.float32, device="cuda") for k in range(order + 1)]
    p = [t.data_ptr() for t in out] + [None] * (2 - order)
    assert lib.gmf_cuda_eval_f32(kind, alpha, n, dX.data_ptr(), *p, None) == 0
    torch.cuda.synchronize()
    got = [t.cpu().numpy().astype(np.float64) for t in out]
    ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X32.astype(np.float64).reshape(n, 9), order, 9)
    return [maxrel(g, r) for g, r in zip(got, ref[1:order + 2])], got, ref


@pytest.mark.parametrize("kind,alpha,name", GMF_KINDS)
@pytest.mark.parametrize("order", [0, 1, 2])
def test_gmf_mixed_c1(kind, alpha, name, order):
    """the four C1 groups (real eigenvalues, rotations, shears, near-confluent shears), rounded to FP32"""
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(16000, seed=5 + order).astype(np.float32)
    errs, got, ref = gmf_errors(kind, alpha, X, order)
    pm = per_matrix(got, ref[1:])
    print(f"mixed gmf {name} order {order}: per call / per matrix " +
          " ".join(f"{n} {e:.2e} / {p:.2e}" for n, e, p in zip("FJH", errs, pm)))
    for g, r in zip(got, ref[1:]):
        assert np.array_equal(np.isnan(g), np.isnan(r))
    assert max(errs) <= GMF_TOL and max(pm) <= GMF_TOL


@pytest.mark.parametrize("kind,alpha,name", GMF_KINDS)
@pytest.mark.parametrize("order", [1, 2])
def test_gmf_mixed_random_general_per_matrix(kind, alpha, name, order):
    """6000 random general matrices rounded to FP32 (diagonalisable, complex pairs, Jordan blocks perturbed by
    1e-14 .. 1e-2, I + 0.5 N): every matrix whose outputs fit FP32 within 1e-6 of the FP64 oracle, NaN exactly where
    the oracle has NaN.  The near-defective ones cancel in the contraction of their record and are recomputed from the
    FP64 record (gmf_kernels.cuh)"""
    X = random_general(1500, seed=99).reshape(-1, 9).astype(np.float32)
    errs, got, ref = gmf_errors(kind, alpha, X, order)
    for g, r in zip(got, ref[1:]):
        assert np.array_equal(np.isnan(g), np.isnan(r))
    pm = per_matrix(got, ref[1:])
    print(f"mixed gmf {name} order {order}, random general: per matrix " + " ".join(f"{n} {p:.2e}" for n, p in
                                                                                   zip("FJH", pm)))
    assert max(pm) <= GMF_TOL


@pytest.mark.parametrize("kind,alpha,name", GMF_KINDS)
def test_gmf_adjoint_f32_random_general_per_matrix(kind, alpha, name):
    """the FP32 adjoints (gmf_cuda_adjoint_f32: Abar = J^T W, J V, W.H.V) on the same random general matrices against
    the FP64 oracle's J and H contracted in FP64: within 1e-6 per matrix where the outputs fit FP32"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    X = random_general(1500, seed=98).reshape(-1, 9).astype(np.float32)
    n = len(X)
    rng = np.random.default_rng(7)
    W = rng.standard_normal((n, 9)).astype(np.float32)
    V = rng.standard_normal((n, 9)).astype(np.float32)
    dA, dW, dV = (torch.from_numpy(a).cuda() for a in (X, W, V))
    outs = [torch.full((n, 9), 7.0, dtype=torch.float32, device="cuda") for _ in range(3)]
    assert lib.gmf_cuda_adjoint_f32(kind, alpha, n, dA.data_ptr(), dW.data_ptr(), dV.data_ptr(), None,
                                    *[t.data_ptr() for t in outs], None) == 0
    torch.cuda.synchronize()
    got = [t.cpu().numpy().astype(np.float64) for t in outs]
    _, _, Jo, Ho = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X.astype(np.float64), 2, 9)
    W64, V64 = W.astype(np.float64), V.astype(np.float64)
    ref = [np.einsum("nm,nmc->nc", W64, Jo.reshape(n, 9, 9)), np.einsum("nmc,nc->nm", Jo.reshape(n, 9, 9), V64),
           np.einsum("nm,nmce,nc->ne", W64, Ho.reshape(n, 9, 9, 9), V64)]
    for g, r in zip(got, ref):
        assert np.array_equal(np.isnan(g), np.isnan(r))
    pm = per_matrix(got, ref)
    print(f"FP32 gmf adjoint {name}, random general: per matrix Abar {pm[0]:.2e} JV {pm[1]:.2e} HWV {pm[2]:.2e}")
    assert max(pm) <= GMF_TOL


@pytest.mark.parametrize("kind,alpha", [(1, 0.0), (2, 0.7)])
@pytest.mark.parametrize("order", [1, 2])
def test_smf_mixed_voigt_store_paths(kind, alpha, order):
    """Voigt orders 1 and 2 write J and H rows by per-entry stores (path 0) or through the TMA unit in boxes of 128-
    or 64-byte rows (paths 1-3; J and H 16-byte aligned, else path 0 runs).  On batch tails around the 32 matrices
    of a warp and the 64 of a CTA every path gives the rows of path 0 to rounding, with the same NaN positions, and
    none writes past row n; path 2 on J and H one float past an aligned address falls back to path 0."""
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    lib = matfun_gb300.load()
    cols = [6, 36, 216][:order + 1]

    def run(X, path, shift):
        n = len(X)
        assert lib.matfun_cuda_smf_f32_tune(order, path) == 0
        dX = torch.from_numpy(np.ascontiguousarray(X)).cuda()
        bufs = [torch.full(((n + 3) * c + 4,), 7.0, dtype=torch.float32, device="cuda") for c in cols]
        views = [b[shift: shift + (n + 3) * c].view(n + 3, c) for b, c in zip(bufs, cols)]
        p = [v.data_ptr() for v in views] + [None] * (2 - order)
        assert (p[1] % 16 == 0) == (shift == 0)
        assert lib.smf_cuda_eval_f32(kind, alpha, n, dX.data_ptr(), *p, None) == 0
        torch.cuda.synchronize()
        for v in views:
            assert bool((v[n:] == 7.0).all()), f"n={n}, path {path}: rows past n written"
        return [v[:n].double().cpu().numpy() for v in views]

    try:
        for n in (1, 7, 31, 32, 33, 63, 64, 65, 97, 129, 1000):
            X = w.c2_smf_spd(n, seed=40 + n)
            if n > 5:
                X[5, 3] = np.nan  # a NaN input row
            ref = run(X, 0, 0)
            for path, shift in ((1, 0), (2, 0), (3, 0), (2, 1)):
                for a, b in zip(run(X, path, shift), ref):
                    assert np.array_equal(np.isnan(a), np.isnan(b)), f"n={n}, path {path}"
                    assert maxrel(a, b) <= 1e-6, f"n={n}, path {path}"
    finally:
        lib.matfun_cuda_smf_f32_tune(order, 2 if order == 1 else 1)  # the library's defaults


@pytest.mark.parametrize("kind,alpha", [(1, 0.0), (2, 0.7)])
def test_smf_mixed_voigt_order0_tails(kind, alpha):
    """Voigt order 0 runs the per-lane kernel (each lane reads its own row and writes its own F row): on batch tails
    around the 32 matrices of a warp and the 64 of a CTA, F equals the F of the matrix layout (the CTA tile) on the
    same matrices to rounding, with the same NaN rows, and nothing past row n is written"""
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    lib = matfun_gb300.load()
    for n in (1, 7, 31, 32, 33, 63, 64, 65, 97, 129, 1000):
        A = w.c2_smf_spd(n, seed=60 + n, as_voigt=False)
        if n > 5:
            A[5, 0, 1] = A[5, 1, 0] = np.nan  # a NaN input row
        X = np.ascontiguousarray(np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], 1))
        F = torch.full((n + 3, 6), 7.0, dtype=torch.float32, device="cuda")
        Fm = torch.full((n, 9), 7.0, dtype=torch.float32, device="cuda")
        dX, dA = torch.from_numpy(X).cuda(), torch.from_numpy(np.ascontiguousarray(A.reshape(n, 9))).cuda()
        assert lib.smf_cuda_eval_f32(kind, alpha, n, dX.data_ptr(), F.data_ptr(), None, None, None) == 0
        assert lib.smf_cuda_eval_matrix_f32(kind, alpha, n, dA.data_ptr(), Fm.data_ptr(), None, None, None) == 0
        torch.cuda.synchronize()
        assert bool((F[n:] == 7.0).all()), f"n={n}: rows past n written"
        got = F[:n].double().cpu().numpy()
        m = Fm.double().cpu().numpy()
        ref = np.stack([m[:, 0], m[:, 4], m[:, 8], m[:, 1], m[:, 2], m[:, 5]], 1)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), f"n={n}"
        assert maxrel(got, ref) <= 1e-6, f"n={n}"


@pytest.mark.parametrize("scale,order", [(1e-30, 0), (1e30, 0), (2.0 ** -20, 2), (2.0 ** 40, 2)])
def test_smf_mixed_extreme_scales(scale, order):
    """the float-float eigensystem scales by a power of two first: matrices of 1e-30 and 1e30 (FP32 range) keep the
    accuracy of unit-scale ones for F; J and H at scales whose values FP32 storage can hold (H of log grows as
    lambda^-2: at condition 1e6 and scale 1e-30 it is far beyond FP32)"""
    from matfun_gb300 import workloads as w
    X = (w.c2_smf_spd(8000, seed=31).astype(np.float64) * scale).astype(np.float32)
    for kind, alpha in ((1, 0.0), (3, 0.0), (2, 0.3)):
        errs, got, ref = errors(False, kind, alpha, X, order)
        for g, r in zip(got, ref[1:]):
            assert np.array_equal(np.isnan(g), np.isnan(r))
        assert max(errs) <= TOL, (kind, errs)


def test_smf_mixed_nonfinite_inputs_give_nan():
    """NaN or infinite input entries: NaN results for that matrix only, the other matrices unaffected"""
    from matfun_gb300 import workloads as w
    X = w.c2_smf_spd(256, seed=32)
    X[3, 0] = np.nan
    X[7, 4] = np.inf
    X[9, 2] = -np.inf
    got = run_f32(False, 1, 0.0, X, 2)
    for g in got:
        assert np.isnan(g[[3, 7, 9]]).all()
        good = np.ones(len(X), bool)
        good[[3, 7, 9]] = False
        assert not np.isnan(g[good]).any()


def run_f32_any(fam, kind, alpha, X32):
    """F, J, H of the FP32 entry point of fam ("smf": smf_cuda_eval_f32 on Voigt vectors, "gmf": gmf_cuda_eval_f32)"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    nf = 6 if fam == "smf" else 9
    n = len(X32)
    dX = torch.from_numpy(np.ascontiguousarray(X32, dtype=np.float32)).cuda()
    out = [torch.full((n, nf ** (k + 1)), 7.0, dtype=torch.float32, device="cuda") for k in range(3)]
    fn = lib.smf_cuda_eval_f32 if fam == "smf" else lib.gmf_cuda_eval_f32
    r = fn(kind, alpha, n, dX.data_ptr(), *[t.data_ptr() for t in out], None)
    torch.cuda.synchronize()
    assert r == 0
    return [t.cpu().numpy().astype(np.float64) for t in out]


@pytest.mark.parametrize("fam", ["smf", "gmf"])
def test_golden_f32(fam):
    """the FP32 golden cases (tests/golden/make_golden_f32.py): the reference's golden inputs rounded to FP32, the
    FP64 oracle's results for those inputs, the FP32 path's per-kind error statement as the per-case tolerance"""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"cases_{fam}_f32.npz"))
    worst = {}
    for kind in np.unique(g["kind"]):
        for alpha in np.unique(g["alpha"][g["kind"] == kind]):
            sel = np.where((g["kind"] == kind) & (g["alpha"] == alpha))[0]
            F, J, H = run_f32_any(fam, int(kind), float(alpha), g["x"][sel])
            for row, i in enumerate(sel):
                for got, name in ((F, "F"), (J, "J"), (H, "H")):
                    ref = g[name][i]
                    assert np.array_equal(np.isnan(got[row]), np.isnan(ref)), f"{fam} case {i} {name}: NaN positions"
                    e = maxrel(got[row], ref)
                    key = (int(kind), float(alpha), name)
                    worst[key] = max(worst.get(key, 0.0), e / g["tol"][i])
    print(f"FP32 golden {fam}, worst error / tolerance: " +
          ", ".join(f"k{k} a{a} {n} {e:.2f}" for (k, a, n), e in sorted(worst.items())))
    assert max(worst.values()) <= 1.0

"""Phase A of the gmf kernels, held against the oracle and the golden cases on the CPU.

The per-matrix record of the general family (scaling, closed-form roots, pair refinement, branch-cut pair, groups, the
confluent group series; F, the real basis r1, r2, the reduced divided differences D2', D3' and the factors sc1, sc2:
matfun_gb300/csrc/gmf_device.cuh) is compiled for the host from the kernels' own header with g++
(tests/host_math/gmf_math_host.cc; host_intrinsics.h supplies the CUDA intrinsics and a one-lane warp vote).  NumPy
then contracts the record into J and H as phase B of the kernels does (r_0 = I, x, y, z = 3a + c):

    J_abcd   = sc1 T4[ac, db],                          T4[x, y]    = sum_mn  r_m[x] D2'_mn r_n[y]
    H_abcdef = sc2 (T6[ac, de, fb] + T6[ae, fc, db]),   T6[x, y, z] = sum_mnp r_m[x] r_n[y] r_p[z] D3'_mnp

Bounds: the FP64 record within 1e-12 of the oracle (as tests/test_parity_gpu.py) and every golden case of the reference
within its own tolerance; the float-float group series of the FP32-storage kernels within 1e-10, four orders of
magnitude below FP32 rounding, on C1 and on the FP32-rounded golden inputs.  Phase B's own arithmetic, the CTA-local
orderings and the device's math library are left to the GPU tests."""
import ctypes
import itertools
import os

import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import build_host_math, maxrel

HERE = os.path.dirname(os.path.abspath(__file__))
KINDS = [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3")]
S2 = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
S3 = [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (0, 0, 2), (0, 1, 2), (1, 1, 2), (0, 2, 2), (1, 2, 2), (2, 2, 2)]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = build_host_math("gmf_math_host.cc", tmp_path_factory.mktemp("host_math"), "-O1")
    if out is None:
        pytest.skip("g++ or the CUDA headers are missing")
    L = ctypes.CDLL(out)
    L.gmf_math.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int64] + \
        [ctypes.c_void_p] * 6
    L.gmf_math.restype = ctypes.c_int
    return L


def record(L, kind, alpha, order, ff, A):
    n = len(A)
    A = np.ascontiguousarray(A, dtype=np.float64).reshape(n, 9)
    F, R12, D2, D3, sc = np.empty((n, 9)), np.empty((n, 18)), np.empty((n, 6)), np.empty((n, 10)), np.empty((n, 2))
    assert L.gmf_math(kind, alpha, order, ff, n, *[x.ctypes.data for x in (A, F, R12, D2, D3, sc)]) == 0
    return F, R12, D2, D3, sc


def contract(order, F, R12, D2, D3, sc):
    """F (n, 9), J (n, 81), H (n, 729) in the layout of gmf_eval, up to the order"""
    n = len(F)
    r = np.empty((n, 3, 3, 3))
    r[:, 0] = np.eye(3)
    r[:, 1], r[:, 2] = R12[:, :9].reshape(n, 3, 3), R12[:, 9:].reshape(n, 3, 3)
    d2 = np.empty((n, 3, 3))
    for k, (a, b) in enumerate(S2):
        d2[:, a, b] = d2[:, b, a] = D2[:, k]
    out = [F]
    if order >= 1:
        T4 = np.einsum("nmac,nmk,nkdb->nacdb", r, d2, r)
        out.append(sc[:, :1] * np.einsum("nacdb->nabcd", T4).reshape(n, 81))
    if order >= 2:
        d3 = np.empty((n, 3, 3, 3))
        for k, t in enumerate(S3):
            for p in set(itertools.permutations(t)):
                d3[:, p[0], p[1], p[2]] = D3[:, k]
        T6 = np.einsum("nmac,nkde,npfb,nmkp->nacdefb", r, r, r, d3, optimize=True)
        H = np.einsum("nacdefb->nabcdef", T6) + np.einsum("naefcdb->nabcdef", T6)
        out.append(sc[:, 1:] * H.reshape(n, 729))
    return out


@pytest.mark.parametrize("kind,alpha,name", KINDS)
@pytest.mark.parametrize("order", [0, 1, 2])
def test_fp64_record_c1(lib, kind, alpha, name, order):
    from matfun_gb300 import workloads as w
    A = w.c1_gmf_groups(2000, seed=3 + order).reshape(-1, 9)
    ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, A, order, 9)[1:order + 2]
    got = contract(order, *record(lib, kind, alpha, order, 0, A))
    errs = [maxrel(g, r) for g, r in zip(got, ref)]
    print(f"gmf phase A on the host, {name}, order {order}: max rel F J H {['%.1e' % e for e in errs]}")
    assert max(errs) <= 1e-12


@pytest.mark.parametrize("kind,alpha,name", KINDS[1:])
def test_ff_series_c1(lib, kind, alpha, name):
    """the float-float group series (log and pow only: exp keeps its split FP64 series in every form)"""
    from matfun_gb300 import workloads as w
    A = w.c1_gmf_groups(2000, seed=9).reshape(-1, 9)
    ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, A, 2, 9)[1:]
    got = contract(2, *record(lib, kind, alpha, 2, 1, A))
    errs = [maxrel(g, r) for g, r in zip(got, ref)]
    print(f"gmf float-float series on the host, {name}: max rel F J H {['%.1e' % e for e in errs]}")
    assert max(errs) <= 1e-10


@pytest.mark.parametrize("fixture,ff,bound", [("cases_gmf.npz", 0, None), ("cases_gmf_f32.npz", 1, 1e-10)])
def test_golden_cases(lib, fixture, ff, bound):
    """every golden gmf case of the reference: the FP64 record within the case's tolerance; the float-float series on
    the FP32-rounded inputs within 1e-10 of the oracle's results for those inputs"""
    g = np.load(os.path.join(HERE, "golden", fixture))
    worst = 0.0
    for kind in np.unique(g["kind"]):
        for alpha in np.unique(g["alpha"][g["kind"] == kind]):
            sel = np.where((g["kind"] == kind) & (g["alpha"] == alpha))[0]
            got = contract(2, *record(lib, int(kind), float(alpha), 2, ff, g["x"][sel].astype(np.float64)))
            for row, i in enumerate(sel):
                for arr, name in zip(got, "FJH"):
                    e = maxrel(arr[row], g[name][i])
                    tol = g["tol"][i] if bound is None else bound
                    worst = max(worst, e / tol)
                    assert e <= tol, f"case {i} (kind {kind}, alpha {alpha}) {name}: {e:.2e} > {tol:.0e}"
    print(f"{fixture}, {'float-float' if ff else 'FP64'} series: worst {worst:.2f} of the bound")


def stress_sets(n, seed=21):
    """general matrices the workloads do not stress: Gaussian (real eigenvalues <= 0: NaN for log, sqrt, pow), Jordan
    blocks of size 3 and 2 perturbed by 1e-4 .. 1e-15, complex pairs at angles up to 3.1415 from the positive axis
    (next to the branch cut), near-singular matrices and matrices scaled by 2^-60 and 2^60; similarity transforms by
    well-conditioned S = N(0, 1) + 3 I"""
    rng = np.random.default_rng(seed)

    def conj(M):
        S = rng.standard_normal((len(M), 3, 3)) + 3 * np.eye(3)
        return S @ M @ np.linalg.inv(S)

    sets = {"gaussian": rng.standard_normal((n, 3, 3)), "gaussian + 3I": rng.standard_normal((n, 3, 3)) + 3 * np.eye(3)}
    for eps in (1e-4, 1e-8, 1e-12, 1e-15):
        c = np.exp(rng.uniform(-1, 1, n))
        J = np.zeros((n, 3, 3))
        J[:, [0, 1, 2], [0, 1, 2]] = c[:, None]
        J[:, 0, 1] = J[:, 1, 2] = 1.0
        sets[f"Jordan 3 + {eps:.0e}"] = conj(J + eps * rng.standard_normal((n, 3, 3)))
        J2 = np.zeros((n, 3, 3))
        J2[:, [0, 1], [0, 1]] = c[:, None]
        J2[:, 0, 1] = 1.0
        J2[:, 2, 2] = np.exp(rng.uniform(-1, 1, n))
        sets[f"Jordan 2 + {eps:.0e}"] = conj(J2 + eps * rng.standard_normal((n, 3, 3)))
    for th in (3.0, 3.14, 3.1415):
        r, t = np.exp(rng.uniform(-1, 1, n)), th * rng.choice([-1.0, 1.0], n)
        M = np.zeros((n, 3, 3))
        M[:, 0, 0] = M[:, 1, 1] = r * np.cos(t)
        M[:, 0, 1], M[:, 1, 0] = -r * np.sin(t), r * np.sin(t)
        M[:, 2, 2] = np.exp(rng.uniform(-1, 1, n))
        sets[f"pair angle {th}"] = conj(M)
    for s in (1e-8, 1e-12):
        D = np.exp(rng.uniform(-1, 1, (n, 3)))
        D[:, 0] = s
        sets[f"near-singular {s:.0e}"] = conj(np.einsum("na,ab->nab", D, np.eye(3)))
    for k in (-60, 60):
        sets[f"scale 2^{k}"] = (rng.standard_normal((n, 3, 3)) + 3 * np.eye(3)) * 2.0 ** k
    return sets


@pytest.mark.parametrize("kind,alpha,name", KINDS + [(2, 2.5, "pow 2.5")])
def test_fp64_record_stress(lib, kind, alpha, name):
    """the FP64 record on the stress sets: within 1e-12 of the oracle per set, NaN exactly where the oracle has NaN"""
    for sname, A in stress_sets(300).items():
        X = A.reshape(-1, 9)
        ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X, 2, 9)[1:]
        got = contract(2, *record(lib, kind, alpha, 2, 0, X))
        for g, r, out in zip(got, ref, "FJH"):
            assert np.array_equal(np.isnan(g), np.isnan(r)), (sname, out)
        if kind == 0 and sname == "scale 2^60":  # exp overflows there in any precision: the same entries overflow
            assert all(np.array_equal(np.isinf(g), np.isinf(r)) for g, r in zip(got, ref)), sname
            continue
        errs = [maxrel(g, r) for g, r in zip(got, ref)]
        assert max(errs) <= 1e-12, (sname, errs)


@pytest.mark.parametrize("kind,alpha,name", KINDS[1:] + [(2, 2.5, "pow 2.5")])
def test_ff_series_stress(lib, kind, alpha, name):
    """the float-float group series of the FP32-storage kernels on the FP32-rounded stress sets: within 1e-10 of the
    oracle's results for the same inputs, NaN exactly where the oracle has NaN"""
    for sname, A in stress_sets(300).items():
        X = A.astype(np.float32).astype(np.float64).reshape(-1, 9)
        ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X, 2, 9)[1:]
        got = contract(2, *record(lib, kind, alpha, 2, 1, X))
        for g, r, out in zip(got, ref, "FJH"):
            assert np.array_equal(np.isnan(g), np.isnan(r)), (sname, out)
        errs = [maxrel(g, r) for g, r in zip(got, ref)]
        assert max(errs) <= 1e-10, (sname, errs)


@pytest.mark.parametrize("kind,alpha,name", KINDS + [(2, 2.5, "pow 2.5")])
def test_ff_series_fp32_constants(lib, kind, alpha, name):
    """the record with the FP32-storage kernels' launch constants (series groups within 0.35 of the centre, series
    ended 2^-44 below the largest term; gmf_coef fp32) on C1, the stress sets and the FP32 golden inputs, all rounded
    to FP32: within 1e-8 of the oracle per call (the FP32 rounding of the record that follows is 6e-8), NaN exactly
    where the oracle has NaN"""
    from matfun_gb300 import workloads as w
    sets = {"C1": w.c1_gmf_groups(2000, seed=9).reshape(-1, 9)}
    sets.update({k: v.reshape(-1, 9) for k, v in stress_sets(200).items()})
    g = np.load(os.path.join(HERE, "golden", "cases_gmf_f32.npz"))
    sel = (g["kind"] == kind) & ((kind != 2) | (g["alpha"] == alpha))
    if sel.any():
        sets["golden f32"] = g["x"][sel]
    for sname, A in sets.items():
        X = np.asarray(A, dtype=np.float32).astype(np.float64)
        ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X, 2, 9)[1:]
        got = contract(2, *record(lib, kind, alpha, 2, 2, X))
        for gg, r, out in zip(got, ref, "FJH"):
            assert np.array_equal(np.isnan(gg), np.isnan(r)), (sname, out)
        if kind == 0 and sname == "scale 2^60":  # exp overflows there in any precision
            continue
        errs = [maxrel(gg, r) for gg, r in zip(got, ref)]
        assert max(errs) <= 1e-8, (sname, errs)


@pytest.fixture(scope="module")
def adj(tmp_path_factory):
    out = build_host_math("gmf_adjoint_host.cc", tmp_path_factory.mktemp("host_math"), "-O1")
    if out is None:
        pytest.skip("g++ or the CUDA headers are missing")
    L = ctypes.CDLL(out)
    for fn in (L.gmf_adjoint_f64, L.gmf_adjoint_f32):
        fn.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int64] + [ctypes.c_void_p] * 7
        fn.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("kind,alpha,name", KINDS)
@pytest.mark.parametrize("f32", [False, True])
def test_adjoint_tile(adj, kind, alpha, name, f32):
    """the general adjoint tile (gmf_adjoint_tile.cuh) run on the CPU: F, Abar = J^T W, JV = J V and HWV = W.H.V
    against the oracle's J and H contracted in FP64, NaN exactly where the oracle has NaN.  FP64: within 1e-12 on C1
    and every stress set (exp: where it is finite).  FP32 (the record folded and rounded once, FP32 contractions):
    within 1e-6 on C1 and 2e-6 on the stress sets within FP32's range (a Jordan block perturbed by 1e-12 and pairs at
    3.14 from the positive axis reach 1.1e-6 .. 1.2e-6); the order-1 launch writes the same F, Abar, JV"""
    from matfun_gb300 import workloads as w
    rng = np.random.default_rng(71)
    sets = {"C1": w.c1_gmf_groups(1000, seed=71).reshape(-1, 9)}
    sets.update({k: v.reshape(-1, 9) for k, v in stress_sets(100).items()})
    dt = np.float32 if f32 else np.float64
    fn = adj.gmf_adjoint_f32 if f32 else adj.gmf_adjoint_f64
    for sname, A in sets.items():
        if (kind == 0 and np.abs(A).max() > 60) or (f32 and sname.startswith("scale")):
            continue
        n = len(A)
        Ac = np.ascontiguousarray(A.astype(dt))
        Wc, Vc = (np.ascontiguousarray(rng.standard_normal((n, 9)).astype(dt)) for _ in range(2))
        _, F, J, H = ol.call(ol.oracle(), "gmf_eval", kind, alpha, Ac.astype(np.float64), 2, 9)
        J4, H5 = J.reshape(n, 9, 9), H.reshape(n, 9, 9, 9)
        W64, V64 = Wc.astype(np.float64), Vc.astype(np.float64)
        ref = [F, np.einsum("nm,nmc->nc", W64, J4), np.einsum("nmc,nc->nm", J4, V64),
               np.einsum("nm,nmce,nc->ne", W64, H5, V64)]
        out = [np.zeros((n, 9), dt) for _ in range(4)]
        assert fn(kind, alpha, n, Ac.ctypes.data, Wc.ctypes.data, Vc.ctypes.data, *[o.ctypes.data for o in out]) == 0
        for o, r in zip(out, ref):
            assert np.array_equal(np.isnan(o), np.isnan(r)), sname
        bound = (1e-6 if sname == "C1" else 2e-6) if f32 else 1e-12
        errs = [maxrel(o, r) for o, r in zip(out, ref)]
        assert max(errs) <= bound, (sname, errs)
        out1 = [np.zeros((n, 9), dt) for _ in range(3)]
        assert fn(kind, alpha, n, Ac.ctypes.data, Wc.ctypes.data, Vc.ctypes.data, *[o.ctypes.data for o in out1],
                  None) == 0
        for a, b in zip(out1, out[:3]):
            assert maxrel(a, b) <= (1e-6 if f32 else 1e-13), sname


@pytest.mark.parametrize("kind,alpha,name", KINDS + [(2, 2.5, "pow 2.5")])
def test_fp64_record_random(lib, kind, alpha, name):
    """the FP64 record per matrix (max error / max |ref| of that matrix's F, J, H) on random general matrices:
    diagonalisable with spectra over e^+-3, complex pairs at random angles, Jordan blocks perturbed by 1e-14 .. 1e-2
    and I + 0.5 N, similarity transforms by S = N(0, 1) + U(0.5, 4) I; within 5e-12 per matrix (last-bit differences
    amplified in H reach 2.5e-12 on 60 000 per kind), NaN exactly where the oracle has NaN"""
    from tests.helpers import maxrel_rows
    rng = np.random.default_rng(99)
    n = 1500

    def conj(M):
        S = rng.standard_normal((len(M), 3, 3)) + rng.uniform(0.5, 4, (len(M), 1, 1)) * np.eye(3)
        return S @ M @ np.linalg.inv(S)

    D = np.zeros((n, 3, 3))
    D[:, [0, 1, 2], [0, 1, 2]] = np.exp(rng.uniform(-3, 3, (n, 3)))
    r, t = np.exp(rng.uniform(-2, 2, n)), rng.uniform(-3.14, 3.14, n)
    M = np.zeros((n, 3, 3))
    M[:, 0, 0] = M[:, 1, 1] = r * np.cos(t)
    M[:, 0, 1], M[:, 1, 0] = -r * np.sin(t), r * np.sin(t)
    M[:, 2, 2] = np.exp(rng.uniform(-2, 2, n))
    J = np.zeros((n, 3, 3))
    J[:, [0, 1, 2], [0, 1, 2]] = np.exp(rng.uniform(-2, 2, n))[:, None]
    J[:, 0, 1], J[:, 1, 2] = rng.uniform(0, 2, n), rng.uniform(0, 2, n)
    J += 10 ** rng.uniform(-14, -2, (n, 1, 1)) * rng.standard_normal((n, 3, 3))
    X = np.concatenate([conj(D), conj(M), conj(J), np.eye(3) + 0.5 * rng.standard_normal((n, 3, 3))]).reshape(-1, 9)
    ref = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X, 2, 9)[1:]
    got = contract(2, *record(lib, kind, alpha, 2, 0, X))
    for g, r_ in zip(got, ref):
        assert np.array_equal(np.isnan(g), np.isnan(r_))
    e = np.max([np.nan_to_num(maxrel_rows(g, r_), nan=0.0) for g, r_ in zip(got, ref)], axis=0)
    assert e.max() <= 5e-12, (name, float(e.max()))


@pytest.mark.parametrize("kind,alpha,name", KINDS)
def test_fp32_record_random(adj, kind, alpha, name):
    """the FP32 form (float-float series, record folded and rounded to FP32 once, FP32 contractions) per matrix on
    6000 random general matrices rounded to FP32 (the families of test_fp64_record_random), through the FP32 adjoint
    tile: F and J^T W with median <= 2e-7 and no matrix beyond 1e-6, NaN exactly where the oracle has NaN.  The
    near-defective matrices, whose contraction cancels (up to 4.5e-4 on 60 000 with the rounded record alone), are
    recomputed from the FP64 record"""
    from tests.helpers import maxrel_rows
    rng = np.random.default_rng(99)
    n = 1500

    def conj(M):
        S = rng.standard_normal((len(M), 3, 3)) + rng.uniform(0.5, 4, (len(M), 1, 1)) * np.eye(3)
        return S @ M @ np.linalg.inv(S)

    D = np.zeros((n, 3, 3))
    D[:, [0, 1, 2], [0, 1, 2]] = np.exp(rng.uniform(-3, 3, (n, 3)))
    r, t = np.exp(rng.uniform(-2, 2, n)), rng.uniform(-3.14, 3.14, n)
    M = np.zeros((n, 3, 3))
    M[:, 0, 0] = M[:, 1, 1] = r * np.cos(t)
    M[:, 0, 1], M[:, 1, 0] = -r * np.sin(t), r * np.sin(t)
    M[:, 2, 2] = np.exp(rng.uniform(-2, 2, n))
    J = np.zeros((n, 3, 3))
    J[:, [0, 1, 2], [0, 1, 2]] = np.exp(rng.uniform(-2, 2, n))[:, None]
    J[:, 0, 1], J[:, 1, 2] = rng.uniform(0, 2, n), rng.uniform(0, 2, n)
    J += 10 ** rng.uniform(-14, -2, (n, 1, 1)) * rng.standard_normal((n, 3, 3))
    X = np.concatenate([conj(D), conj(M), conj(J), np.eye(3) + 0.5 * rng.standard_normal((n, 3, 3))])
    X = np.ascontiguousarray(X.reshape(-1, 9).astype(np.float32))
    N = len(X)
    W = np.ascontiguousarray(rng.standard_normal((N, 9)).astype(np.float32))
    _, F, Jm, _ = ol.call(ol.oracle(), "gmf_eval", kind, alpha, X.astype(np.float64), 1, 9)
    ref = [F, np.einsum("nm,nmc->nc", W.astype(np.float64), Jm.reshape(N, 9, 9))]
    out = [np.zeros((N, 9), np.float32) for _ in range(2)]
    assert adj.gmf_adjoint_f32(kind, alpha, N, X.ctypes.data, W.ctypes.data, W.ctypes.data, out[0].ctypes.data,
                               out[1].ctypes.data, None, None) == 0
    for o, r_ in zip(out, ref):
        assert np.array_equal(np.isnan(o), np.isnan(r_))
    e = np.max([np.nan_to_num(maxrel_rows(o.astype(np.float64), r_), nan=0.0) for o, r_ in zip(out, ref)], axis=0)
    assert np.median(e) <= 2e-7 and e.max() <= 1e-6, (name, np.median(e), e.max())

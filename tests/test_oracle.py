"""The CPU oracle (oracle/oracle.c) against the reference's golden vectors (tests/golden, from testdata/cases*.txt of
the reference) and, where it was built here, against the reference's own compiled CPU library."""
import os

import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel

HERE = os.path.dirname(os.path.abspath(__file__))


def golden(fam):
    return np.load(os.path.join(HERE, "golden", f"cases_{fam}.npz"))


@pytest.mark.parametrize("fam,fn,nf", [("smf", "smf_eval", 6), ("gmf", "gmf_eval", 9)])
def test_oracle_matches_golden(fam, fn, nf):
    g = golden(fam)
    assert len(g["kind"]) == (210 if fam == "smf" else 204)
    worst = 0.0
    for i in range(len(g["kind"])):
        r, F, J, H = ol.call(ol.oracle(), fn, int(g["kind"][i]), float(g["alpha"][i]), g["x"][i:i + 1], 2, nf)
        assert r == 0
        for got, name in ((F, "F"), (J, "J"), (H, "H")):
            e = maxrel(got, g[name][i])
            worst = max(worst, e / g["tol"][i])
            assert e <= g["tol"][i], f"{fam} case {i} {name}: {e:.2e} > {g['tol'][i]:.0e}"
    assert worst < 1.0


def test_oracle_matrix_layout_matches_golden():
    """smf matrix layout: the golden Voigt cases expanded with the layout weights (matfun.h:17-25)"""
    from tests.helpers import voigt_to_matrix
    g = golden("smf")
    midx = [0, 3, 4, 3, 1, 5, 4, 5, 2]
    wt = np.array([1.0 if m % 4 == 0 else 0.5 for m in range(9)])
    for i in range(0, len(g["kind"]), 7):
        A = voigt_to_matrix(g["x"][i:i + 1])
        r, F, J, H = ol.call(ol.oracle(), "smf_eval_matrix", int(g["kind"][i]), float(g["alpha"][i]),
                             A.reshape(1, 9), 2, 9)
        assert r == 0
        Fv, Jv, Hv = g["F"][i], g["J"][i].reshape(6, 6), g["H"][i].reshape(6, 6, 6)
        Fm = Fv[midx]
        Jm = Jv[np.ix_(midx, midx)] * wt[None, :]
        Hm = Hv[np.ix_(midx, midx, midx)] * wt[None, :, None] * wt[None, None, :]
        tol = g["tol"][i]
        assert maxrel(F, Fm) <= tol and maxrel(J, Jm) <= tol and maxrel(H, Hm) <= tol


def _random_inputs(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, 3, 3))
    A = B @ B.transpose(0, 2, 1) + 0.5 * np.eye(3)
    G = 0.3 * rng.standard_normal((n, 3, 3)) + 1.5 * np.eye(3)
    return A, G


@pytest.mark.skipif(ol.reference() is None, reason="reference library not built here (needs the reference sources)")
@pytest.mark.parametrize("kind,alpha", [(0, 0.0), (1, 0.0), (3, 0.0), (2, 0.3), (2, 1.7), (2, 60.5)])
def test_oracle_bitwise_equals_reference_library(kind, alpha):
    from matfun_gb300 import workloads as w
    A, G = _random_inputs(2000, 11 + kind)
    V = w.voigt(A)
    G = np.concatenate([G, w.c1_gmf_groups(2000, seed=3)])
    V = np.concatenate([V, w.c0_smf_spd(2000, seed=4)])
    ref = ol.reference()
    for fam, X, nf in (("smf_eval", V, 6), ("smf_eval_matrix", A.reshape(-1, 9), 9), ("gmf_eval", G.reshape(-1, 9), 9)):
        a = ol.call(ol.oracle(), fam, kind, alpha, X, 2, nf)
        b = ol.call(ref, fam, kind, alpha, X, 2, nf)
        assert a[0] == b[0]
        for x, y in zip(a[1:], b[1:]):
            assert np.array_equal(np.isnan(x), np.isnan(y))
            assert maxrel(x, y) <= 1e-15, (fam, kind, alpha)


def test_oracle_error_codes():
    X = np.eye(3).reshape(1, 9).repeat(4, 0)
    o = ol.oracle()
    assert ol.call(o, "gmf_eval", 9, 0.0, X, 0, 9)[0] == -1
    assert ol.call(o, "gmf_eval", 2, 0.0, X, 0, 9)[0] == -1
    assert ol.call(o, "gmf_eval", 2, -1.0, X, 0, 9)[0] == -1
    Y = X.copy()
    Y[2, 1] += 0.1  # not symmetric: -3, NaN for that matrix only
    r, F, _, _ = ol.call(o, "smf_eval_matrix", 0, 0.0, Y, 0, 9)
    assert r == -3 and np.isnan(F[2]).all() and np.isfinite(F[[0, 1, 3]]).all()


def test_oracle_domain_nan():
    """gmf: a real eigenvalue <= 0 gives NaN for log / sqrt / pow only, in that matrix only"""
    G = np.stack([np.eye(3), np.diag([-1.0, 2.0, 3.0]), 1.5 * np.eye(3)]).reshape(3, 9)
    for kind, alpha in ((0, 0.0), (1, 0.0), (3, 0.0), (2, 0.3)):
        r, F, J, H = ol.call(ol.oracle(), "gmf_eval", kind, alpha, G, 2, 9)
        assert r == 0
        assert np.isnan(F[1]).all() == (kind != 0)
        assert np.isfinite(F[[0, 2]]).all()


@pytest.mark.parametrize("fam,fn,nf", [("smf", "smf_eval", 6), ("gmf", "gmf_eval", 9)])
def test_fp32_golden_fixtures_reproduce(fam, fn, nf):
    """tests/golden/cases_*_f32.npz (tests/golden/make_golden_f32.py): the expected values are the oracle's F, J, H
    of the stored FP32 inputs (a sample of every kind, 1e-14: another host's libm may differ in the last bits), and
    every tolerance is the stated one of its kind"""
    import importlib.util
    here = os.path.dirname(os.path.abspath(__file__))
    g = np.load(os.path.join(here, "golden", f"cases_{fam}_f32.npz"))
    spec = importlib.util.spec_from_file_location("make_golden_f32", os.path.join(here, "golden", "make_golden_f32.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    assert g["x"].dtype == np.float32
    for i in range(len(g["kind"])):
        assert g["tol"][i] == mk.tol(fam, int(g["kind"][i]), float(g["alpha"][i]))
    for kind in np.unique(g["kind"]):
        for i in np.where(g["kind"] == kind)[0][:6]:
            r, F, J, H = ol.call(ol.oracle(), fn, int(kind), float(g["alpha"][i]), g["x"][i:i + 1].astype(np.float64),
                                 2, nf)
            assert r == 0
            for got, name in ((F, "F"), (J, "J"), (H, "H")):
                assert np.array_equal(np.isnan(got[0]), np.isnan(g[name][i]))
                assert maxrel(got[0], g[name][i]) <= 1e-14, (fam, i, name)

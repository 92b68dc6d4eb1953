"""Parity of the CUDA library (through its C ABI) with the oracle and the reference's golden vectors:
every family x kind x order, odd batch sizes, NaN positions, error codes.  Tolerance: max |x - ref| / max |ref|
<= 1e-12 per call (FP64 path), the per-case tolerance of the golden files, NaN exactly where the oracle has NaN."""
import os

import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel, voigt_to_matrix

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-12
KINDS = [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3"), (2, 1.7, "pow 1.7")]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import matfun_gb300
    matfun_gb300.load()


def _gpu(*a, **k):
    from tests.gpu_util import gpu_call
    return gpu_call(*a, **k)


def _cmp(fam, kind, alpha, X, order, nf, tol=TOL):
    g = _gpu(fam, kind, alpha, X, order, nf)
    o = ol.call(ol.oracle(), fam, kind, alpha, X, order, nf)
    assert g[0] == 0
    worst = 0.0
    for a, b in zip(g[1:1 + order + 1], o[1:1 + order + 1]):
        assert np.array_equal(np.isnan(a), np.isnan(b)), f"{fam} kind {kind}: NaN positions differ"
        worst = max(worst, maxrel(a, b))
    assert worst <= tol, f"{fam} kind {kind} al {alpha} order {order}: max rel {worst:.2e}"
    return g, o


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, 3, 3))
    return B @ B.transpose(0, 2, 1) + 0.5 * np.eye(3)


@pytest.mark.parametrize("fam,fn,nf", [("smf", "smf_eval", 6), ("gmf", "gmf_eval", 9)])
def test_golden_cases(fam, fn, nf):
    g = np.load(os.path.join(HERE, "golden", f"cases_{fam}.npz"))
    kinds = g["kind"]
    for kind in np.unique(kinds):
        for alpha in np.unique(g["alpha"][kinds == kind]):
            sel = np.where((kinds == kind) & (g["alpha"] == alpha))[0]
            r, F, J, H = _gpu(fn, int(kind), float(alpha), g["x"][sel], 2, nf)
            assert r == 0
            for row, i in enumerate(sel):
                for got, name in ((F, "F"), (J, "J"), (H, "H")):
                    e = maxrel(got[row], g[name][i])
                    assert e <= g["tol"][i], f"{fam} case {i} (kind {kind}, al {alpha}) {name}: {e:.2e}"


def test_golden_smf_matrix_layout():
    g = np.load(os.path.join(HERE, "golden", "cases_smf.npz"))
    for kind in np.unique(g["kind"]):
        for alpha in np.unique(g["alpha"][g["kind"] == kind]):
            sel = np.where((g["kind"] == kind) & (g["alpha"] == alpha))[0]
            A = voigt_to_matrix(g["x"][sel]).reshape(-1, 9)
            _cmp("smf_eval_matrix", int(kind), float(alpha), A, 2, 9, tol=float(g["tol"][sel].max()))


@pytest.mark.parametrize("kind,alpha,name", KINDS)
@pytest.mark.parametrize("order", [0, 1, 2])
def test_smf_random_spd(kind, alpha, name, order):
    A = _spd(1000, 7)
    A[17, 0, 1] += 0.1  # one non-symmetric matrix: NaN on the device (the CPU returns -3)
    V = np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], 1)
    _cmp("smf_eval", kind, alpha, V, order, 6)
    g = _gpu("smf_eval_matrix", kind, alpha, A.reshape(-1, 9), order, 9)
    o = ol.call(ol.oracle(), "smf_eval_matrix", kind, alpha, A.reshape(-1, 9), order, 9)
    assert g[0] == 0 and o[0] == -3
    assert np.isnan(g[1][17]).all() and np.isnan(o[1][17]).all()
    for a, b in zip(g[1:order + 2], o[1:order + 2]):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert maxrel(a, b) <= TOL


@pytest.mark.parametrize("kind,alpha,name", KINDS)
@pytest.mark.parametrize("order", [0, 1, 2])
def test_gmf_random_general(kind, alpha, name, order):
    rng = np.random.default_rng(8)
    G = 0.3 * rng.standard_normal((1000, 3, 3)) + 1.5 * np.eye(3)
    G[3] = [[1, 0.7, 0], [0, 1, 0], [0, 0, 1]]            # defective (shear)
    G[4] = [[0.6, -0.8, 0], [0.8, 0.6, 0], [0, 0, 1.2]]   # rotation block (complex pair)
    G[5] = np.diag([-1.0, 2.0, 3.0])                      # outside the domain of log / sqrt / pow
    g, o = _cmp("gmf_eval", kind, alpha, G.reshape(-1, 9), order, 9)
    assert np.isnan(g[1][5]).all() == (kind != 0)


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 63, 64, 65, 127, 129, 1000])
def test_batch_tails(n):
    """every tail of the 64-matrix CTA tile, for each family at order 2 (also checks nothing is written past n)"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    rng = np.random.default_rng(n)
    G = (0.3 * rng.standard_normal((n, 3, 3)) + 1.5 * np.eye(3)).reshape(n, 9)
    _cmp("gmf_eval", 1, 0.0, G, 2, 9)
    V = np.stack([x.ravel()[[0, 4, 8, 1, 2, 5]] for x in _spd(n, n)])
    _cmp("smf_eval", 2, 0.3, V, 2, 6)
    # guard band: outputs of n + 64 matrices, the last 64 must keep their sentinel
    dA = torch.from_numpy(np.concatenate([G, G[:1].repeat(64, 0)])).cuda()
    dF = torch.full((n + 64, 9), 3.25, dtype=torch.float64, device="cuda")
    dJ = torch.full((n + 64, 81), 3.25, dtype=torch.float64, device="cuda")
    dH = torch.full((n + 64, 729), 3.25, dtype=torch.float64, device="cuda")
    r = lib.gmf_cuda_eval(1, 0.0, n, dA.data_ptr(), dF.data_ptr(), dJ.data_ptr(), dH.data_ptr(), None)
    torch.cuda.synchronize()
    assert r == 0
    for t in (dF, dJ, dH):
        assert bool((t[n:] == 3.25).all())


def test_configs_sampled():
    """the benchmark workloads (smf SPD with repeated eigenvalues; gmf real / rotation / shear / near-confluent
    groups) on a sample, every kind of the benchmark metric"""
    from matfun_gb300 import workloads as w
    V = w.c0_smf_spd(8192, seed=0)
    _cmp("smf_eval", 1, 0.0, V, 2, 6)
    G = w.c1_gmf_groups(8192, seed=1).reshape(-1, 9)
    for kind, alpha in ((0, 0.0), (1, 0.0), (3, 0.0)):
        _cmp("gmf_eval", kind, alpha, G, 2, 9)


def test_error_codes_and_grid_limit():
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    n = 1000
    d = torch.zeros(n * 9, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    assert lib.gmf_cuda_eval(9, 0.0, n, p, p, None, None, None) == -1
    assert lib.gmf_cuda_eval(2, 0.0, n, p, p, None, None, None) == -1
    assert lib.gmf_cuda_eval(0, 0.0, n, p, p, None, p, None) == -1
    assert lib.gmf_cuda_eval(0, 0.0, 0, p, p, None, None, None) == 0
    assert lib.smf_cuda_eval(9, 0.0, n, p, p, None, None, None) == -1
    assert lib.smf_cuda_eval(2, 0.0, n, p, p, None, None, None) == -1
    assert lib.smf_cuda_eval(0, 0.0, n, p, p, None, p, None) == -1
    assert lib.smf_cuda_eval_matrix(0, 0.0, -1, p, p, None, None, None) == -1
    assert lib.smf_cuda_eval(0, 0.0, 0, p, p, None, None, None) == 0
    # grids the reference cannot launch: -2 without a launch, and no pending CUDA error afterwards
    assert lib.smf_cuda_eval(0, 0.0, (2**31 - 1) * 32 + 1, p, p, None, None, None) == -2
    assert lib.smf_cuda_eval(0, 0.0, 1 << 40, p, p, None, None, None) == -2
    assert lib.gmf_cuda_eval(0, 0.0, (2**31 - 1) * 64 + 1, p, p, None, None, None) == -2
    torch.cuda.synchronize()
    x = torch.ones(4, dtype=torch.float64, device="cuda") * 2
    assert float(x.sum()) == 8.0


def test_streams_and_python_api():
    """the torch front end queues on the current stream; results equal the direct C ABI call"""
    import torch

    import matfun_gb300
    rng = np.random.default_rng(3)
    G = 0.3 * rng.standard_normal((500, 3, 3)) + np.eye(3)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        F, J, H = matfun_gb300.gmf("log", torch.from_numpy(G).cuda(), order=2)
    s.synchronize()
    Fo, Jo, Ho = ol.gmf("log", G, order=2)
    assert F.shape == (500, 3, 3) and J.shape == (500, 3, 3, 3, 3) and H.shape == (500,) + (3,) * 6
    assert maxrel(H.cpu().numpy(), Ho) <= TOL and maxrel(F.cpu().numpy(), Fo) <= TOL
    Fs = matfun_gb300.smf("sqrt", torch.from_numpy(_spd(10, 1)).cuda())
    assert maxrel(Fs.cpu().numpy(), ol.smf("sqrt", _spd(10, 1))) <= TOL


@pytest.mark.parametrize("kind,alpha,name", [(0, 0.0, "exp"), (1, 0.0, "log"), (3, 0.0, "sqrt"), (2, 0.3, "pow 0.3")])
@pytest.mark.parametrize("order", [1, 2])
def test_gmf_ordered_launch(kind, alpha, name, order):
    """n >= 2^15: the launch ordered by spectral class (key, scan, scatter, the ordered evaluation and the plain
    evaluation of the last rows, whose share of J or H held the scratch) against the oracle on the whole batch"""
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(36000, seed=31).reshape(-1, 9)
    _cmp("gmf_eval", kind, alpha, X, order, 9)


@pytest.mark.parametrize("kind,alpha,name", [(0, 0.0, "exp"), (1, 0.0, "log"), (2, 0.3, "pow 0.3")])
@pytest.mark.parametrize("mat", [False, True])
def test_smf_ordered_launch(kind, alpha, name, mat):
    """n >= 2^17, order 2: the smf launch ordered by the branch pattern of the second divided differences (key,
    scan, scatter, the ordered evaluation and the plain evaluation of the last rows, whose share of H held the
    scratch) against the oracle on the whole batch; in the matrix layout one non-symmetric matrix gives NaN"""
    from matfun_gb300 import workloads as w
    n = (1 << 17) + 77
    if mat:
        A = w.c0_smf_spd(n, seed=41, as_voigt=False)
        A[n - 5, 0, 2] += 1.0  # in the plain tail
        A[1000, 1, 2] += 1.0   # in the ordered part
        g, _ = _cmp("smf_eval_matrix", kind, alpha, A.reshape(n, 9), 2, 9)
        assert np.isnan(g[1][n - 5]).all() and np.isnan(g[1][1000]).all()
    else:
        _cmp("smf_eval", kind, alpha, w.c0_smf_spd(n, seed=41), 2, 6)

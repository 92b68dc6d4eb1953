"""The host-buffer entry points (smf/gmf_cuda_eval_host) and the reference-named libmatfun.so (smf_eval,
smf_eval_matrix, gmf_eval on host arrays, with the GPU behind them): results equal the oracle's, -3 for a
non-symmetric matrix in smf_eval_matrix exactly as the reference CPU library, batches that span several chunks,
pageable and page-locked host arrays."""
import ctypes
import os

import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def shim():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.zeros(1, device="cuda")
    return ol._load(os.path.join(ROOT, "matfun_gb300", "libmatfun.so"), "")


@pytest.mark.parametrize("order", [0, 1, 2])
def test_gmf_eval_host_across_chunks(shim, order):
    from matfun_gb300 import workloads as w
    n = (1 << 16) + 37 if order == 2 else (1 << 18) + 5
    X = w.c1_gmf_groups(n, seed=9).reshape(n, 9)
    idx = np.r_[0:300, n - 300:n, (1 << 16) - 40:(1 << 16) + 40]
    idx = idx[idx < n]
    g = ol.call(shim, "gmf_eval", 1, 0.0, X, order, 9)
    o = ol.call(ol.oracle(), "gmf_eval", 1, 0.0, X[idx], order, 9)
    assert g[0] == 0
    for a, b in zip(g[1:order + 2], o[1:order + 2]):
        assert np.array_equal(np.isnan(a[idx]), np.isnan(b))
        assert maxrel(a[idx], b) <= 1e-12


@pytest.mark.parametrize("kind,alpha", [(0, 0.0), (1, 0.0), (3, 0.0), (2, 0.3)])
def test_smf_eval_matrix_host_codes(shim, kind, alpha):
    rng = np.random.default_rng(kind)
    B = rng.standard_normal((3000, 3, 3))
    A = B @ B.transpose(0, 2, 1) + 0.5 * np.eye(3)
    A[1234, 2, 0] += 0.1
    g = ol.call(shim, "smf_eval_matrix", kind, alpha, A.reshape(-1, 9), 2, 9)
    o = ol.call(ol.oracle(), "smf_eval_matrix", kind, alpha, A.reshape(-1, 9), 2, 9)
    assert g[0] == -3 and o[0] == -3
    for a, b in zip(g[1:], o[1:]):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert maxrel(a, b) <= 1e-12
    V = np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], 1)
    g = ol.call(shim, "smf_eval", kind, alpha, V, 1, 6)
    o = ol.call(ol.oracle(), "smf_eval", kind, alpha, V, 1, 6)
    assert g[0] == 0 and maxrel(g[2], o[2]) <= 1e-12
    # symmetric input again: the asymmetry count starts from zero on every call
    A[1234, 2, 0] -= 0.1
    assert ol.call(shim, "smf_eval_matrix", kind, alpha, A.reshape(-1, 9), 0, 9)[0] == 0


def test_pinned_buffers_and_names(shim):
    import torch
    lib = ctypes.CDLL(os.path.join(ROOT, "matfun_gb300", "libmatfun.so"))
    lib.smf_simd_name.restype = ctypes.c_char_p
    assert lib.smf_simd_name() == b"cuda-sm_103a"
    from matfun_gb300 import workloads as w
    n = 5000
    X = torch.from_numpy(w.c1_gmf_groups(n, seed=2).reshape(n, 9)).pin_memory()
    F = torch.empty((n, 9), dtype=torch.float64).pin_memory()
    J = torch.empty((n, 81), dtype=torch.float64).pin_memory()
    H = torch.empty((n, 729), dtype=torch.float64).pin_memory()
    import matfun_gb300
    r = matfun_gb300.load().gmf_cuda_eval_host(0, 0.0, n, X.data_ptr(), F.data_ptr(), J.data_ptr(), H.data_ptr())
    assert r == 0
    o = ol.call(ol.oracle(), "gmf_eval", 0, 0.0, X.numpy(), 2, 9)
    assert maxrel(H.numpy(), o[3]) <= 1e-12 and maxrel(F.numpy(), o[1]) <= 1e-12


@pytest.mark.parametrize("fam", ["smf_matrix", "gmf"])
def test_in_place_path_equals_chunked_copies(shim, fam):
    """every array page-locked: the kernels read and write host memory in place over the host link; the results are
    those of the chunked copy path (pageable arrays) -- bit for bit for smf; for gmf to 1e-13, since the device path
    orders a batch by spectral class and a warp's neighbours can change the last bits of a series -- and -3 for a
    non-symmetric matrix as there"""
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    lib = matfun_gb300.load()
    n = (1 << 16) + 123
    if fam == "gmf":
        A = w.c1_gmf_groups(4 * ((n + 3) // 4), seed=21)[:n].reshape(n, 9)
        fn, code = lib.gmf_cuda_eval_host, 0
    else:
        A = w.c0_smf_spd(n, seed=21, as_voigt=False).reshape(n, 9)
        A[777, 2] += 0.5  # not symmetric: -3 and NaN results for that matrix
        fn, code = lib.smf_cuda_eval_matrix_host, -3
    outs = {}
    for pinned in (True, False):
        tens = [torch.from_numpy(np.ascontiguousarray(A))] + [torch.full((n, k), 3.0, dtype=torch.float64)
                                                               for k in (9, 81, 729)]
        if pinned:
            tens = [t.pin_memory() for t in tens]
        assert fn(1, 0.0, n, *[t.data_ptr() for t in tens]) == code
        outs[pinned] = [t.numpy() for t in tens[1:]]
    for a, b in zip(outs[True], outs[False]):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        if fam == "gmf":
            assert maxrel(a, b) <= 1e-13
        else:
            assert np.array_equal(np.nan_to_num(a), np.nan_to_num(b))

"""Parity with the reference's own CUDA kernels (its cuda/src/matfun_cuda.cu compiled for sm_103a from its sources,
oracle/_ref/matfun_cuda_ref.cubin): same device buffers, every kind and order, max rel <= 1e-12 and identical NaN
positions.  Skipped where the cubin was not built (it needs the reference sources)."""
import numpy as np
import pytest

from tests import ref_gpu
from tests.helpers import maxrel

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not ref_gpu.available(), reason="reference cubin not built here")]


def _run_both(fam, kind, alpha, X, order):
    import torch

    import matfun_gb300
    lib, ref = matfun_gb300.load(), ref_gpu.load()
    nf = 6 if fam == "smf" else 9
    n = len(X)
    dX = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    outs = []
    for impl in ("ours", "ref"):
        F = torch.full((n, nf), 5.0, dtype=torch.float64, device="cuda")
        J = torch.full((n, nf * nf), 5.0, dtype=torch.float64, device="cuda")
        H = torch.full((n, nf ** 3), 5.0, dtype=torch.float64, device="cuda")
        p = [F.data_ptr(), J.data_ptr() if order else None, H.data_ptr() if order > 1 else None]
        if impl == "ours":
            fn = lib.smf_cuda_eval if fam == "smf" else lib.gmf_cuda_eval
            r = fn(kind, alpha, n, dX.data_ptr(), *p, None)
        else:
            fn = ref.refgpu_smf if fam == "smf" else ref.refgpu_gmf
            r = fn(kind, alpha, order, n, dX.data_ptr(), *p, None)
        torch.cuda.synchronize()
        assert r == 0, (impl, r)
        outs.append([t.cpu().numpy() for t in (F, J, H)][:order + 1])
    return outs


@pytest.mark.parametrize("kind,alpha", [(0, 0.0), (1, 0.0), (3, 0.0), (2, 0.3), (2, 1.7)])
@pytest.mark.parametrize("order", [0, 1, 2])
def test_gmf_matches_reference_kernel(kind, alpha, order):
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(4096, seed=5).reshape(-1, 9)
    ours, ref = _run_both("gmf", kind, alpha, X, order)
    for a, b in zip(ours, ref):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert maxrel(a, b) <= 1e-12


@pytest.mark.parametrize("kind,alpha", [(0, 0.0), (1, 0.0), (3, 0.0), (2, 0.3), (2, 1.7)])
@pytest.mark.parametrize("order", [0, 1, 2])
def test_smf_matches_reference_kernel(kind, alpha, order):
    from matfun_gb300 import workloads as w
    X = w.c0_smf_spd(4096, seed=6)
    ours, ref = _run_both("smf", kind, alpha, X, order)
    for a, b in zip(ours, ref):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert maxrel(a, b) <= 1e-12

"""Size-independent properties at the benchmark's full size (gmf order 2 on n = 2^20 general matrices; smf order 2
on n = 65536 SPD matrices): exact index symmetries of H and J, a sampled comparison with the oracle, exp(log A) = A,
and NaN-freeness inside the domain."""
import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel_rows

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from matfun_gb300 import workloads as w
    return w.c1_gmf_groups(1 << 20, seed=1)


def test_gmf_log_full_size(c1):
    import torch

    import matfun_gb300
    A = torch.from_numpy(c1).cuda()
    F, J, H = matfun_gb300.gmf("log", A, order=2)
    torch.cuda.synchronize()
    n = A.shape[0]
    # NaN only for matrices outside the domain (a real eigenvalue <= 0: some rotations and random matrices), and
    # then for the whole matrix; none in the shear groups
    bad = torch.isnan(F).any(dim=(1, 2))
    assert bool((torch.isnan(H).flatten(1).all(1) == bad).all())
    assert int(bad[n // 2:].sum()) == 0 and int(bad.sum()) < n // 50
    # H_abcdef = H_abefcd exactly (the two index pairs of the second derivative)
    Hp = H.permute(0, 1, 2, 5, 6, 3, 4)
    assert bool(((H == Hp) | (torch.isnan(H) & torch.isnan(Hp))).all())
    # a sample against the oracle, one from each group of the workload
    idx = np.concatenate([np.arange(g * n // 4, g * n // 4 + 512) for g in range(4)])
    Fo, Jo, Ho = ol.gmf("log", c1[idx], order=2)
    for got, ref in ((F, Fo), (J, Jo), (H, Ho)):
        g = got[idx].reshape(len(idx), -1).cpu().numpy()
        assert np.array_equal(np.isnan(g), np.isnan(ref.reshape(len(idx), -1)))
        e = maxrel_rows(g, ref.reshape(len(idx), -1))
        assert e.max() <= 1e-12, e.max()
    # exp(log A) = A on the random group (inside the domain)
    ok = ~bad[: n // 4]
    E = matfun_gb300.gmf("exp", F[: n // 4][ok])
    err = (E - A[: n // 4][ok]).abs().amax() / A[: n // 4][ok].abs().amax()
    assert float(err) <= 1e-12


def test_smf_log_full_size():
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    V = w.c0_smf_spd(65536, seed=0)
    F, J, H = matfun_gb300.smf("log", torch.from_numpy(V).cuda(), order=2)
    torch.cuda.synchronize()
    Hn = H.cpu().numpy()
    assert np.array_equal(Hn, Hn.transpose(0, 1, 3, 2))  # H_i,pq = H_i,qp exactly
    idx = np.arange(0, 65536, 61)
    Fo, Jo, Ho = ol.smf("log", V[idx], order=2)
    for got, ref in ((F, Fo), (J, Jo), (H, Ho)):
        e = maxrel_rows(got[idx].reshape(len(idx), -1).cpu().numpy(), ref.reshape(len(idx), -1))
        assert e.max() <= 1e-12, e.max()

"""matfun_gb300.host, the NumPy front end on the GPU (the reference's matfun.smf / matfun.gmf on host arrays):
argument errors on the CPU; on the GPU the values of the oracle, the reference's shapes, ValueError for a
non-symmetric matrix, pageable and page-locked outputs."""
import numpy as np
import pytest

from tests import oracle_lib as ol
from tests.helpers import maxrel


def test_arguments_rejected_like_the_reference():
    from matfun_gb300 import host
    A = np.eye(3)[None]
    for bad in (lambda: host.smf("cos", A), lambda: host.gmf("pow", A), lambda: host.gmf("pow", A, alpha=-1.0),
                lambda: host.smf("exp", A, order=3), lambda: host.smf("exp", np.zeros((4, 5))),
                lambda: host.gmf("log", np.zeros((4, 6)))):
        with pytest.raises(ValueError):
            bad()


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [False, True])
def test_values_shapes_and_errors(pinned):
    from matfun_gb300 import host
    from matfun_gb300 import workloads as w
    A = w.c1_gmf_groups(400, seed=12).reshape(4, 100, 3, 3)
    F, J, H = host.gmf("log", A, order=2, pinned=pinned)
    assert F.shape == (4, 100, 3, 3) and J.shape == (4, 100) + (3,) * 4 and H.shape == (4, 100) + (3,) * 6
    o = ol.gmf("log", A.reshape(-1, 3, 3), order=2)
    for got, ref in zip((F, J, H), o):
        got = got.reshape(ref.shape)
        assert np.array_equal(np.isnan(got), np.isnan(ref)) and maxrel(got, ref) <= 1e-12
    V = w.c0_smf_spd(300, seed=12)
    Fv, Jv = host.smf("pow", V, alpha=0.3, order=1, pinned=pinned)
    assert Fv.shape == (300, 6) and Jv.shape == (300, 6, 6)
    ro = ol.smf("pow", V, alpha=0.3, order=1)
    assert maxrel(Fv, ro[0]) <= 1e-12 and maxrel(Jv.reshape(ro[1].shape), ro[1]) <= 1e-12
    S = w.c0_smf_spd(50, seed=13, as_voigt=False)
    assert maxrel(host.smf("exp", S, pinned=pinned), ol.smf("exp", S)) <= 1e-12
    S[7, 0, 1] += 1.0
    with pytest.raises(ValueError, match="symmetric"):
        host.smf("exp", S, pinned=pinned)

"""The C ABI library (no GPU needed): it loads, exports every function include/*.h declares, and the Python
front end checks its arguments like the reference's NumPy API.  No compute call is made here."""
import glob
import os

import numpy as np
import pytest

from tests.helpers import header_functions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import matfun_gb300
    if not os.path.exists(matfun_gb300.library_path()):
        from matfun_gb300 import build
        build.build_cuda()
    return matfun_gb300.load()


def test_headers_declare_the_reference_entry_points():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names |= set(header_functions(h))
    assert {"smf_cuda_eval", "smf_cuda_eval_matrix", "gmf_cuda_eval"} <= names


# which in-tree library implements each public header
HEADER_LIBRARY = {"matfun_cuda.h": "libmatfun_cuda.so", "matfun.h": "libmatfun.so"}


def test_library_exports_every_declared_symbol(lib):
    import ctypes

    from matfun_gb300 import build
    build.build_shim()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        so = HEADER_LIBRARY[os.path.basename(h)]
        handle = ctypes.CDLL(os.path.join(ROOT, "matfun_gb300", so))
        for name in header_functions(h):
            assert hasattr(handle, name), f"{name} declared in {os.path.basename(h)} but not exported by {so}"


def test_host_entry_points_reject_bad_arguments_without_device(lib):
    """argument errors of the host-buffer forms come back before any CUDA call"""
    assert lib.gmf_cuda_eval_host(9, 0.0, 10, None, None, None, None) == -1
    assert lib.smf_cuda_eval_host(2, 0.0, 10, None, None, None, None) == -1
    assert lib.smf_cuda_eval_matrix_host(0, 0.0, -5, None, None, None, None) == -1
    assert lib.gmf_cuda_eval_host(0, 0.0, 0, None, None, None, None) == 0


def test_version(lib):
    assert b"sm_103a" in lib.matfun_cuda_version()


def test_argument_checks_before_any_device_work():
    import matfun_gb300
    import torch
    A = torch.zeros(4, 3, 3, dtype=torch.float64)
    with pytest.raises(ValueError):
        matfun_gb300.gmf("cosh", A)
    with pytest.raises(ValueError):
        matfun_gb300.gmf("pow", A)
    with pytest.raises(ValueError):
        matfun_gb300.smf("exp", A, order=3)
    with pytest.raises(TypeError):
        matfun_gb300.gmf("exp", A)  # host tensor: the device interface refuses it


def test_abi_error_codes_need_no_device(lib):
    """invalid arguments are rejected on the host before any CUDA call (null pointers are never dereferenced)"""
    assert lib.gmf_cuda_eval(9, 0.0, 10, None, None, None, None, None) == -1
    assert lib.gmf_cuda_eval(2, 0.0, 10, None, None, None, None, None) == -1
    assert lib.smf_cuda_eval(0, 0.0, -1, None, None, None, None, None) == -1
    assert lib.smf_cuda_eval(0, 0.0, 0, None, None, None, None, None) == 0
    assert lib.smf_cuda_eval(0, 0.0, 10, None, None, None, None, None) == -1  # null input with n > 0
    # the tangent entry point: invalid kind, pow without alpha, n < 0, no A or no K for n > 0; empty batch
    assert lib.gmf_cuda_tangent(4, 0.0, 10, None, None, None, None, None) == -1
    assert lib.gmf_cuda_tangent(2, -1.0, 10, None, None, None, None, None) == -1
    assert lib.gmf_cuda_tangent(1, 0.0, -3, None, None, None, None, None) == -1
    assert lib.gmf_cuda_tangent(1, 0.0, 10, None, None, None, None, None) == -1
    assert lib.gmf_cuda_tangent(1, 0.0, 0, None, None, None, None, None) == 0


def test_workloads_shapes_and_spectra():
    from matfun_gb300 import workloads as w
    V = w.c0_smf_spd(4000, seed=0)
    assert V.shape == (4000, 6)
    from tests.helpers import voigt_to_matrix
    lam = np.linalg.eigvalsh(voigt_to_matrix(V))
    assert (lam > 0).all()
    gaps = np.minimum(lam[:, 1] - lam[:, 0], lam[:, 2] - lam[:, 1]) / lam[:, 2]
    frac_rep = np.mean(gaps < 1e-12)
    assert 0.08 < frac_rep < 0.16
    G = w.c1_gmf_groups(4000, seed=1)
    assert G.shape == (4000, 3, 3)
    ev = np.linalg.eigvals(G[1000:2000])
    assert (np.abs(ev.imag).max(axis=1) > 1e-6).mean() > 0.9  # rotations: complex pairs

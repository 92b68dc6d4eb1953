"""matfun_cuda_batched_noalloc -- the batched launch for callers that cannot allocate device memory (a framework
that owns every device allocation, a plugin handed only device arrays).  Its request table lives in a fixed array of
device memory inside the library instead of a buffer from cudaMalloc.  Checked through the C ABI against
matfun_cuda_batched (same results to rounding, identical NaN positions) on two calls in a row -- the second call
reuses the array the first one left behind -- and the clear error for a table larger than the array.  Kept in the
last file pytest collects, so that a failure here cannot hide the results of the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import matfun_gb300
    torch.zeros(1, device="cuda")
    return matfun_gb300.load()


def _requests(seed):
    import torch

    from matfun_gb300 import batched
    from matfun_gb300 import workloads as w
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(18):
        fam = ["gmf", "smf_voigt", "smf"][i % 3]
        kind = ["log", "exp", "sqrt", "pow"][i % 4]
        n = int(rng.integers(1, 1500))
        x = w.c1_gmf_groups(max(n, 4), seed=seed + i)[:n] if fam == "gmf" else \
            w.c0_smf_spd(n, seed=seed + i, as_voigt=fam == "smf_voigt")
        t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        if fam != "gmf" and i % 2:
            t = t.float()
        reqs.append(batched.request(fam, kind, t, order=i % 3, alpha=0.3 if kind == "pow" else None))
    # a gmf log order-2 request large enough (>= 2048 matrices) that matfun_cuda_batched orders it by spectral class,
    # which the no-allocation form, having no room for the permutation, evaluates in its given order
    t = torch.from_numpy(w.c1_gmf_groups(3000, seed=seed)).cuda()
    reqs.append(batched.request("gmf", "log", t, order=2))
    return reqs


def _outputs(reqs):
    return [[t.clone() for t in (r.F, r.J, r.H) if t is not None] for r in reqs]


def _close(a, b):
    import torch
    if not torch.equal(torch.isnan(a), torch.isnan(b)):
        return False
    g, e = torch.nan_to_num(a.double()), torch.nan_to_num(b.double())
    tol = 1e-13 if a.dtype == torch.float64 else 1e-6
    return float((g - e).abs().max()) <= tol * max(float(e.abs().max()), 1e-300)


def test_noalloc_matches_batched_on_two_calls(lib):
    import torch

    from matfun_gb300 import batched
    reqs = _requests(11)
    arr = batched._array(reqs)
    assert lib.matfun_cuda_batched(ctypes.cast(arr, ctypes.c_void_p), len(reqs), None) == 0
    torch.cuda.synchronize()
    expected = _outputs(reqs)
    for call in range(2):
        for r in reqs:
            for t in (r.F, r.J, r.H):
                if t is not None:
                    t.fill_(float("nan") if call == 0 else -3.0)
        assert lib.matfun_cuda_batched_noalloc(ctypes.cast(arr, ctypes.c_void_p), len(reqs), None) == 0
        torch.cuda.synchronize()
        for got, exp in zip(_outputs(reqs), expected):
            for a, b in zip(got, exp):
                assert _close(a, b), f"call {call + 1}"


def test_noalloc_allocates_no_device_memory(lib):
    """after a first call on the device, further calls leave the device's free memory and torch's allocations as
    they were"""
    import torch

    from matfun_gb300 import batched
    reqs = _requests(13)
    arr = batched._array(reqs)
    assert lib.matfun_cuda_batched_noalloc(ctypes.cast(arr, ctypes.c_void_p), len(reqs), None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    used0 = torch.cuda.memory_allocated()
    for _ in range(3):
        assert lib.matfun_cuda_batched_noalloc(ctypes.cast(arr, ctypes.c_void_p), len(reqs), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == used0


def test_noalloc_refuses_a_capturing_stream(lib):
    """the table is copied from host memory that lives only during the call, so a stream being captured into a CUDA
    graph is refused (-1) with nothing queued"""
    import torch

    from matfun_gb300 import batched
    reqs = _requests(17)[:3]
    arr = batched._array(reqs)
    st = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(st):
        with torch.cuda.graph(g, stream=st):
            r = lib.matfun_cuda_batched_noalloc(ctypes.cast(arr, ctypes.c_void_p), len(reqs),
                                                ctypes.c_void_p(st.cuda_stream))
            torch.zeros(1, device="cuda")  # (a node, so that the graph is not empty)
    assert r == -1
    torch.cuda.synchronize()


def test_noalloc_rejects_a_table_beyond_its_array(lib):
    import torch

    from matfun_gb300 import batched
    eye = torch.eye(3, dtype=torch.float64, device="cuda")[None]
    many = [batched.request("gmf", "log", 2.0 * eye, order=0) for _ in range(200)]
    arr = batched._array(many)  # 200 gmf requests need about 500 KB of table, more than the 256 KiB array
    assert lib.matfun_cuda_batched_noalloc(ctypes.cast(arr, ctypes.c_void_p), len(many), None) == -4
    assert lib.matfun_cuda_batched_noalloc(ctypes.cast(arr, ctypes.c_void_p), 50, None) == 0
    torch.cuda.synchronize()
    log2 = float(np.log(2.0))
    for r in many[:50]:
        assert torch.allclose(r.F, log2 * eye.reshape(1, 9), rtol=1e-15, atol=1e-15)

"""The batched persistent kernel: many requests of mixed family / kind / order / precision in one launch give
the results of the single entry points (to rounding: the tile routines are compiled separately, 1e-13 relative
for FP64 and 1e-6 for FP32, identical NaN positions); a plan replays under CUDA-graph capture; invalid requests are
rejected before anything runs; the autotuner stores and applies a choice."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def mixed_requests(seed, count=40, nmax=3000):
    import torch

    from matfun_gb300 import batched
    from matfun_gb300 import workloads as w
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        fam = ["smf_voigt", "smf", "gmf"][i % 3]
        kind = ["exp", "log", "sqrt", "pow"][rng.integers(4)]
        order = int(rng.integers(3))
        f32 = rng.uniform() < 0.4
        n = int(rng.integers(1, nmax))
        if fam == "gmf":
            x = w.c1_gmf_groups(max(n, 4), seed=seed + i)[:n]
        else:
            x = w.c0_smf_spd(n, seed=seed + i, as_voigt=fam == "smf_voigt")
        t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        t = t.float() if f32 else t
        reqs.append(batched.request(fam, kind, t, order=order, alpha=0.3 if kind == "pow" else None))
    return reqs


def same(got, exp):
    import torch
    nan_ok = torch.equal(torch.isnan(got), torch.isnan(exp))
    g, e = torch.nan_to_num(got.double(), nan=0.0), torch.nan_to_num(exp.double(), nan=0.0)
    tol = 1e-13 if got.dtype == torch.float64 else 1e-6
    return nan_ok and float((g - e).abs().max()) <= tol * max(float(e.abs().max()), 1e-300)


def single(r):
    """the same request through its single entry point"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    c = r.c
    fn = {(0, 0): lib.smf_cuda_eval, (1, 0): lib.smf_cuda_eval_matrix, (2, 0): lib.gmf_cuda_eval,
          (0, 1): lib.smf_cuda_eval_f32, (1, 1): lib.smf_cuda_eval_matrix_f32,
          (2, 1): lib.gmf_cuda_eval_f32}[(c.family, c.dtype)]
    outs = [torch.empty_like(t) if t is not None else None for t in (r.F, r.J, r.H)]
    p = lambda t: None if t is None else t.data_ptr()
    assert fn(c.kind, c.alpha, c.n, r.x.data_ptr(), *map(p, outs), None) == 0
    return outs


def test_batched_equals_single_entry_points():
    import torch

    from matfun_gb300 import batched
    reqs = mixed_requests(1)
    batched.run(reqs)
    torch.cuda.synchronize()
    for r in reqs:
        ref = single(r)
        torch.cuda.synchronize()
        for got, exp in zip((r.F, r.J, r.H), ref):
            if exp is not None:
                assert same(got, exp), (r.c.family, r.c.kind, r.c.order, r.c.dtype)


def test_plan_graph_capture_and_replay():
    import torch

    from matfun_gb300 import batched
    reqs = mixed_requests(2, count=24)
    plan = batched.Plan(reqs)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run()  # warm-up outside the capture (sets the kernel's shared-memory attribute)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    for r in reqs:
        r.F.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for r in reqs:
        ref = single(r)
        torch.cuda.synchronize()
        assert same(r.F, ref[0])


def test_invalid_requests_rejected():
    import ctypes

    import torch

    import matfun_gb300
    from matfun_gb300 import batched
    lib = matfun_gb300.load()
    reqs = mixed_requests(3, count=3)
    bad = batched.request("gmf", "pow", torch.eye(3, dtype=torch.float64, device="cuda")[None], order=1, alpha=1.0)
    bad.c.alpha = -1.0
    arr = batched._array(reqs + [bad])
    assert lib.matfun_cuda_batched(ctypes.cast(arr, ctypes.c_void_p), 4, None) == -1
    bad.c.alpha = 1.0
    bad.c.J = None  # order 1 without J
    arr = batched._array([bad])
    assert lib.matfun_cuda_batched(ctypes.cast(arr, ctypes.c_void_p), 1, None) == -1
    f32bad = batched.request("gmf", "log", torch.eye(3, device="cuda")[None], order=0)
    f32bad.c.dtype = 2  # neither FP64 nor FP32
    assert lib.matfun_cuda_batched(ctypes.cast(batched._array([f32bad]), ctypes.c_void_p), 1, None) == -1
    assert lib.matfun_cuda_batched(None, 0, None) == 0
    assert lib.matfun_cuda_batched_tune(0, 1) == -1 and lib.matfun_cuda_batched_tune(2, 1) == 0


def test_autotune_roundtrip(tmp_path, monkeypatch):
    from matfun_gb300 import autotune
    monkeypatch.setenv("MATFUN_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    reqs = mixed_requests(4, count=12, nmax=2000)
    best, times = autotune.tune(reqs, reps=1, candidates=[{"ctas_per_sm": 1, "longest_first": 1},
                                                          {"ctas_per_sm": 2, "longest_first": 1}])
    assert best in ({"ctas_per_sm": 1, "longest_first": 1}, {"ctas_per_sm": 2, "longest_first": 1})
    assert autotune.apply(reqs) == best

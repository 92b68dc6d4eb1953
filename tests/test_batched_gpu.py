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


@pytest.fixture
def smf_tile(request):
    """the smf tile geometry of the batched tables built during one test (128 restored afterwards)"""
    import matfun_gb300
    lib = matfun_gb300.load()
    assert lib.matfun_cuda_batched_tune_tiles(request.param) == 0
    yield request.param
    lib.matfun_cuda_batched_tune_tiles(128)


@pytest.mark.parametrize("smf_tile", [128, 64], indirect=True)
def test_batched_equals_single_entry_points(smf_tile):
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
    assert lib.matfun_cuda_batched_tune_tiles(32) == -1 and lib.matfun_cuda_batched_tune_tiles(128) == 0


def test_autotune_roundtrip(tmp_path, monkeypatch):
    from matfun_gb300 import autotune
    monkeypatch.setenv("MATFUN_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    reqs = mixed_requests(4, count=12, nmax=2000)
    cands = [{"ctas_per_sm": 1, "longest_first": 1, "smf_tile": 128},
             {"ctas_per_sm": 2, "longest_first": 1, "smf_tile": 64}]
    best, times = autotune.tune(reqs, reps=1, candidates=cands)
    assert best in cands and len(times) == 2
    assert autotune.apply(reqs) == best
    autotune._set(autotune.load(), autotune.DEFAULT)  # later tests run with the default tuning


@pytest.mark.parametrize("smf_tile", [128, 64], indirect=True)
def test_batched_c3_mix_against_oracle(smf_tile):
    """a C3-style mix in one persistent launch held directly against the FP64 oracle: every family, kind and order,
    FP64 and FP32 requests, and gmf log / pow requests of >= 2048 matrices that the launch orders by spectral class
    first; FP64 within 1e-12 per call with NaN exactly where the oracle has NaN, FP32 per matrix within the bounds of
    tests/test_mixed_gpu.py (1e-6; smf H 2.5e-6) against the oracle on the FP32 values"""
    import torch

    from matfun_gb300 import batched
    from matfun_gb300 import workloads as w
    from tests import oracle_lib as ol
    from tests.helpers import maxrel, maxrel_rows_fp32
    rng = np.random.default_rng(23)
    reqs, meta = [], []
    plan = [("gmf", "log", 2, False, 4000), ("gmf", "pow", 2, False, 2500), ("gmf", "log", 2, True, 3000),
            ("gmf", "sqrt", 1, True, 2200), ("gmf", "exp", 2, False, 900)]
    for i in range(15):
        plan.append((["smf_voigt", "smf", "gmf"][i % 3], ["exp", "log", "sqrt", "pow"][i % 4], i % 3, bool(i % 2),
                     int(rng.integers(1, 1500))))
    for fam, kind, order, f32, n in plan:
        x = w.c1_gmf_groups(max(n, 4), seed=n)[:n] if fam == "gmf" else \
            w.c0_smf_spd(n, seed=n, as_voigt=fam == "smf_voigt")
        t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        t = t.float() if f32 else t
        alpha = 0.3 if kind == "pow" else None
        reqs.append(batched.request(fam, kind, t, order=order, alpha=alpha))
        meta.append((fam, kind, order, f32, alpha))
    batched.run(reqs)
    torch.cuda.synchronize()
    cfam = {"smf_voigt": ("smf_eval", 6), "smf": ("smf_eval_matrix", 9), "gmf": ("gmf_eval", 9)}
    for r, (fam, kind, order, f32, alpha) in zip(reqs, meta):
        fn, nf = cfam[fam]
        X = r.x.double().cpu().numpy().reshape(r.n, -1)
        ref = ol.call(ol.oracle(), fn, ol.KINDS[kind], alpha or 0.0, X, order, nf)[1:order + 2]
        for name, got, exp in zip("FJH", (r.F, r.J, r.H), ref):
            g = got.double().cpu().numpy()
            assert np.array_equal(np.isnan(g), np.isnan(exp)), (fam, kind, order, f32, name)
            if f32:
                bound = 2.5e-6 if (fam != "gmf" and name == "H") else 1e-6
                e = float(np.max(maxrel_rows_fp32(g, exp), initial=0.0))
            else:
                bound, e = 1e-12, maxrel(g, exp)
            assert e <= bound, (fam, kind, order, f32, name, e)

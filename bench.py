"""Benchmark: gmf log, order 2 (F, J, H), FP64, n = 2^20 general 3x3 matrices in the four groups of the reference's
workload (real spectra, rotations with stretch, shears, near-confluent shears), through the C ABI of
libmatfun_cuda (gmf_cuda_eval).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--kind log] [--n 1048576]

One JSON line on rank 0.  `value` is whole-job matrices/s with inputs resident in HBM (CUDA events on the launching
stream; the per-step traffic of 6.9 GB is far above the 126 MB L2, so no flush is needed); `e2e` is the same metric
through the host-buffer C ABI (gmf_cuda_eval_host, the reference's gmf_eval signature on host arrays) from page-locked
HOST arrays, with all host-device copies inside the timed region (host wall clock around the synchronous call).  Multi-GPU
(torchrun): every rank evaluates its own n matrices (independent matrices, no collective on the data path).
--impl reference times the CPU implementation of the same path on the host cores (the reference's compiled library
where it was built, otherwise the oracle restatement of it), on bounded samples of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

KINDS = {"exp": 0, "log": 1, "pow": 2, "sqrt": 3}
BYTES_PER_MATRIX = {0: 72 + 72, 1: 72 + 72 + 648, 2: 72 + 72 + 648 + 5832}  # FP64 in + F (+ J) (+ H)
METRIC = "gmf log order-2 matrices/s (FP64)"
# FP64 floating-point operations per matrix of one order-2 call on this workload (2 per DFMA): the ordered gmf_kernel
# <LOG, 2> (DFMA 2355, DADD 1006, DMUL 723) plus gmf_key_kernel (the closed-form roots: 144, 64, 76), from the ncu
# counters smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum at n = 262144
FP64_FLOP_PER_MATRIX = {"log": 2 * (2355 + 144) + (1006 + 64) + (723 + 76)}
# DRAM bytes per matrix of the ordered gmf_kernel<LOG, 2> launch from one ncu capture at n = 262144 on the same
# workload (101.4 MB read + 1752.0 MB written for 259 584 matrices; the algorithmic bytes are 6624 per matrix, the
# extra reads are the partial sectors at the ends of the rows the ordered launch scatters)
NCU_DRAM_BYTES_PER_MATRIX = (101.44e6 + 1752.03e6) / 259584


def launches_per_call(kind, n):
    """kernels one order-2 gmf_cuda_eval call launches: key, scan, scatter, the ordered launch and the tail launch
    (every kind with 2^15 <= n <= 2^31 - 1), else one plain launch"""
    return 5 if (1 << 15) <= n <= (1 << 31) - 1 else 1


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region"""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def section(out, name, fn):
    """an auxiliary part of the JSON line: a failure is recorded under its name (the exception's text) instead of
    ending the run, so that the headline measured before it and the CPU baseline still print"""
    try:
        out[name] = fn()
    except Exception as e:
        out[name] = {"error": f"{type(e).__name__}: {e}"}


def dist_setup(n_gpus):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device="cuda"):
    """the slowest rank's value (the job ends with its last rank); nccl on the GPUs, gloo on CPU tensors"""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(n_per_rank, ms, world):
    """matrices/s of the whole job: every rank evaluates its own n_per_rank matrices (weak scaling, no collective on
    the data path), the job takes the slowest rank's time"""
    return world * n_per_rank / (ms * 1e-3)


def rank_seed(rank):
    """the seed of a rank's matrices: independent replicas of the workload"""
    return 1 + rank


def cpu_rate(kind_code, alpha, X, order, budget_s=10.0):
    """matrices/s of the CPU implementation over repeated calls on X until budget_s has elapsed; (rate, cores, kind)"""
    from tests import oracle_lib as ol
    ref = ol.reference()
    lib, kind = (ref, "reference") if ref is not None else (ol.oracle(), "port")
    ol.call(lib, "gmf_eval", kind_code, alpha, X[:256], order, 9)  # warm-up
    done, t0 = 0, time.perf_counter()
    while True:
        ol.call(lib, "gmf_eval", kind_code, alpha, X, order, 9)
        done += len(X)
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return done / el, cores, kind, done


def run_reference(args, rank, world):
    """--impl reference: the CPU path on this host's cores, rank 0 only"""
    if rank != 0:
        return
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(args.n, seed=1).reshape(-1, 9)
    sample = min(len(X), args.cpu_sample)
    # a bounded sample covering all four groups
    idx = np.concatenate([np.arange(g * len(X) // 4, g * len(X) // 4 + sample // 4) for g in range(4)])
    Xs = np.ascontiguousarray(X[idx])
    from tests import oracle_lib as ol
    ref = ol.reference()
    lib, kind = (ref, "reference") if ref is not None else (ol.oracle(), "port")
    for _ in range(args.warmup):
        ol.call(lib, "gmf_eval", KINDS[args.kind], args.alpha, Xs[:1024], 2, 9)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ol.call(lib, "gmf_eval", KINDS[args.kind], args.alpha, Xs, 2, 9)
    el = time.perf_counter() - t0
    rate = args.steps * len(Xs) / el
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    out = {"metric": METRIC.replace("log", args.kind), "value": rate, "unit": "matrices/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": f"gmf {args.kind} order 2, general 3x3, four groups (random / rotation / shear / "
                                  f"near-confluent), seed 1", "n": args.n, "sample_per_step": len(Xs)},
           "cpu_baseline": {"value": rate, "unit": "matrices/s", "cores": cores, "kind": kind,
                            "sample": f"{len(Xs)} matrices per step (equal parts of the four groups), OpenMP"},
           "e2e": {"value": rate, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def _mixed_pair(x32, nf, fn32, fn64, steps, dev, kind=1, alpha=0.0, order=2):
    """time the FP32 entry point and the FP64 one (default: log, order 2) on the same values; max relative error of
    the FP32 results against the FP64 ones (max-norm per output array) on a sample of 65536 matrices"""
    import torch
    n = x32.shape[0]
    d32 = x32.to(dev)
    d64 = d32.double()
    outs = {}
    for tag, dt, x, fn in (("f32", torch.float32, d32, fn32), ("f64", torch.float64, d64, fn64)):
        F = torch.empty((n, nf), dtype=dt, device=dev)
        J = torch.empty((n, nf ** 2), dtype=dt, device=dev) if order >= 1 else None
        H = torch.empty((n, nf ** 3), dtype=dt, device=dev) if order >= 2 else None
        p = lambda t: None if t is None else t.data_ptr()
        call = lambda: fn(kind, alpha, n, x.data_ptr(), p(F), p(J), p(H), None)
        for _ in range(2):
            assert call() == 0
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            call()
        e1.record()
        e1.synchronize()
        outs[tag] = (e0.elapsed_time(e1) / steps, F, J, H)
        del F, J, H
    idx = torch.arange(0, n, max(1, n // 65536), device=dev)
    err = {}
    for k, name in ((1, "F"), (2, "J"), (3, "H"))[:order + 1]:
        a, b = outs["f32"][k][idx].double(), outs["f64"][k][idx]
        both = torch.isnan(a) & torch.isnan(b)
        d = torch.where(both, torch.zeros_like(a), (a - b).abs())
        err[name] = float(d.max() / torch.nan_to_num(b, nan=0.0).abs().max())
    return outs["f32"][0], outs["f64"][0], err, int(idx.numel())


def mixed_vs_fp64(lib, args, dev, hbm):
    """smf log order 2 (Voigt) on the C2 workload (n = 2^24 SPD, condition number log-uniform in [1, 1e6], smallest
    eigenvalue gap log-uniform in [1e-12, 1], stored as FP32): the mixed-precision path (FP32 storage and bulk
    arithmetic) against the FP64 path on the same values, with the max relative error of the mixed results against
    the FP64 results on a sample"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.mixed_n
    x32 = torch.from_numpy(w.c2_smf_spd(n, seed=2))
    ms32, ms64, err, ns = _mixed_pair(x32, 6, lib.smf_cuda_eval_f32, lib.smf_cuda_eval, args.mixed_steps, dev)
    bytes32 = (6 + 6 + 36 + 216) * 4
    return {"workload": f"smf log order 2, Voigt, n={n} SPD, condition log-uniform [1,1e6], smallest gap "
                        "log-uniform [1e-12,1], FP32 storage (C2)",
            "mixed_matrices_per_s": n / (ms32 * 1e-3), "fp64_matrices_per_s": n / (ms64 * 1e-3),
            "speedup_vs_fp64": ms64 / ms32, "mixed_ms": ms32, "fp64_ms": ms64,
            "max_rel_err_vs_fp64": err, "err_sample": ns,
            "mixed_hbm_frac": bytes32 * n / (ms32 * 1e-3) / 1e9 / hbm, "bytes_per_matrix_fp32": bytes32}


def mixed_sweep(lib, args, dev, hbm):
    """the C2 workload over every kind and order (smf Voigt, n = 2^24 SPD stored as FP32; pow with one exponent
    alpha ~ U(0.1, 0.9) per call, seeded): the mixed-precision path against the FP64 path on the same values"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.mixed_n
    x32 = torch.from_numpy(w.c2_smf_spd(n, seed=2))
    rng = np.random.default_rng(2)
    rows = []
    for name, kind in (("exp", 0), ("log", 1), ("sqrt", 3), ("pow", 2)):
        alpha = float(rng.uniform(0.1, 0.9)) if kind == 2 else 0.0
        for order in (0, 1, 2):
            ms32, ms64, err, ns = _mixed_pair(x32, 6, lib.smf_cuda_eval_f32, lib.smf_cuda_eval, args.mixed_steps,
                                              dev, kind, alpha, order)
            b32 = 4 * (6 + (6, 42, 258)[order])
            rows.append({"kind": name, "alpha": alpha, "order": order, "mixed_matrices_per_s": n / (ms32 * 1e-3),
                         "fp64_matrices_per_s": n / (ms64 * 1e-3), "speedup_vs_fp64": ms64 / ms32,
                         "mixed_hbm_frac": b32 * n / (ms32 * 1e-3) / 1e9 / hbm, "max_rel_err_vs_fp64": err})
            torch.cuda.empty_cache()
    return {"workload": f"C2: smf Voigt, n={n} SPD, condition log-uniform [1,1e6], smallest gap log-uniform "
                        "[1e-12,1], FP32 storage; every kind and order", "err_sample": ns, "rows": rows}


def mixed_gmf_vs_fp64(lib, args, dev, hbm):
    """gmf log order 2 on the C1 workload (n = 2^20, the four groups), stored as FP32: the mixed-precision gmf path
    (FP64 spectral analysis and series, FP32 storage and J / H assembly) against the FP64 path on the same values"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.gmf_mixed_n
    x32 = torch.from_numpy(w.c1_gmf_groups(n, seed=1).astype(np.float32).reshape(n, 9))
    ms32, ms64, err, ns = _mixed_pair(x32, 9, lib.gmf_cuda_eval_f32, lib.gmf_cuda_eval, args.mixed_steps, dev)
    bytes32 = (9 + 9 + 81 + 729) * 4
    return {"workload": f"gmf log order 2, n={n} general matrices (C1 groups), FP32 storage",
            "mixed_matrices_per_s": n / (ms32 * 1e-3), "fp64_matrices_per_s": n / (ms64 * 1e-3),
            "speedup_vs_fp64": ms64 / ms32, "mixed_ms": ms32, "fp64_ms": ms64,
            "max_rel_err_vs_fp64": err, "err_sample": ns,
            "mixed_hbm_frac": bytes32 * n / (ms32 * 1e-3) / 1e9 / hbm, "bytes_per_matrix_fp32": bytes32}


def smf_c0(lib, args, dev):
    """C0: smf log order 2 on Voigt vectors, FP64 (n = 65536 SPD matrices with 10 % repeated and 2 % triple
    eigenvalues), through smf_cuda_eval; batches of 2^17 or more run the ordered launch"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.smf_n
    V = torch.from_numpy(w.c0_smf_spd(n)).to(dev)
    F, J, H = (torch.empty((n, k), dtype=torch.float64, device=dev) for k in (6, 36, 216))
    call = lambda: lib.smf_cuda_eval(1, 0.0, n, V.data_ptr(), F.data_ptr(), J.data_ptr(), H.data_ptr(), None)
    for _ in range(3):
        assert call() == 0
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(args.steps, 10)
    e0.record()
    for _ in range(steps):
        call()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"workload": f"C0: smf log order 2, Voigt, n={n} SPD (10 % repeated, 2 % triple eigenvalues), FP64",
            "ms": ms, "matrices_per_s": n / (ms * 1e-3), "ordered": n >= (1 << 17)}


def tangent_vs_materialised(lib, args, dev):
    """the tangent of psi(A) = |log A|^2 / 2 (G = J^T F, K = J^T J + F : H) on the C1 workload, n = 2^20 FP64: the
    fused kernel (gmf_cuda_tangent, no J or H formed) against evaluating F, J, H (gmf_cuda_eval) and contracting them
    with torch (bmm / einsum), with the max relative difference of the two on the whole batch"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.n
    A = torch.from_numpy(w.c1_gmf_groups(n, seed=1).reshape(n, 9)).to(dev)
    F, G, K = (torch.empty((n, k), dtype=torch.float64, device=dev) for k in (9, 9, 81))
    Fe, Je, He = (torch.empty((n, k), dtype=torch.float64, device=dev) for k in (9, 81, 729))
    st = torch.cuda.current_stream().cuda_stream

    def fused():
        assert lib.gmf_cuda_tangent(1, 0.0, n, A.data_ptr(), F.data_ptr(), G.data_ptr(), K.data_ptr(), st) == 0

    def unfused():
        assert lib.gmf_cuda_eval(1, 0.0, n, A.data_ptr(), Fe.data_ptr(), Je.data_ptr(), He.data_ptr(), st) == 0
        Jm = Je.view(n, 9, 9)
        Gu = torch.bmm(Fe.view(n, 1, 9), Jm).view(n, 9)
        Ku = torch.bmm(Jm.transpose(1, 2), Jm) + torch.bmm(Fe.view(n, 1, 9), He.view(n, 9, 81)).view(n, 9, 9)
        return Gu, Ku

    def timed(fn, steps):
        for _ in range(2):
            out = fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            out = fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / steps, out

    t_f, _ = timed(fused, 3)
    t_u, (Gu, Ku) = timed(unfused, 3)

    def rel(a, b):
        d = torch.where(torch.isnan(a) & torch.isnan(b), torch.zeros_like(a), (a - b).abs())
        return float(d.max() / torch.nan_to_num(b, nan=0.0).abs().max())

    return {"workload": f"psi(A) = |log A|^2 / 2 on C1, n={n} FP64: F, G = J^T F, K = J^T J + F : H",
            "fused_matrices_per_s": n / (t_f * 1e-3), "fused_ms": t_f,
            "materialised_matrices_per_s": n / (t_u * 1e-3), "materialised_ms": t_u, "speedup": t_u / t_f,
            "bytes_written_per_matrix": {"fused": 8 * (9 + 9 + 81), "materialised": 8 * (9 + 81 + 729) + 8 * 90},
            "max_rel_diff_G": rel(G, Gu), "max_rel_diff_K": rel(K, Ku.reshape(n, 81))}


def adjoint_vs_materialised(lib, args, dev):
    """C4: the gradient of L = sum <W, f(A)> and its Hessian-vector product along V, for smf log (SPD, the C0
    generator) and gmf pow 0.3 (real and rotation groups of C1), n = 2^22 FP64: the adjoint kernels (no J, H formed)
    against evaluating J (resp. H) with the eval kernels and contracting it with W (resp. W and V)"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.adj_n
    res = {}
    for fam, kind, alpha in (("smf", 1, 0.0), ("gmf", 2, 0.3)):
        if fam == "smf":
            A = torch.from_numpy(w.c0_smf_spd(n, seed=4, as_voigt=False)).to(dev)
        else:
            A = torch.from_numpy(w.c1_gmf_groups(2 * n, seed=4)[: n]).to(dev)
        g = torch.Generator(device=dev).manual_seed(5)
        W = torch.randn(A.shape, dtype=torch.float64, device=dev, generator=g)
        V = torch.randn(A.shape, dtype=torch.float64, device=dev, generator=g)
        Abar, HWV, JV = torch.empty_like(A), torch.empty_like(A), torch.empty_like(A)
        fn = lib.smf_cuda_adjoint if fam == "smf" else lib.gmf_cuda_adjoint
        ev = lib.smf_cuda_eval_matrix if fam == "smf" else lib.gmf_cuda_eval
        vjp = lambda: fn(kind, alpha, n, A.data_ptr(), W.data_ptr(), None, None, Abar.data_ptr(), None, None, None)
        hvp = lambda: fn(kind, alpha, n, A.data_ptr(), W.data_ptr(), V.data_ptr(), None, None, JV.data_ptr(),
                         HWV.data_ptr(), None)

        def timeit(f, reps=3):
            assert f() in (0, None)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                f()
            e1.record()
            e1.synchronize()
            return e0.elapsed_time(e1) / reps

        t_vjp, t_hvp = timeit(vjp), timeit(hvp)
        # materialised: J (and H) by the eval kernel in chunks of at most 2^20, then the contractions
        ch = min(1 << 20, n)
        Fm = torch.empty((ch, 9), dtype=torch.float64, device=dev)
        Jm = torch.empty((ch, 81), dtype=torch.float64, device=dev)
        Hm = torch.empty((ch, 729), dtype=torch.float64, device=dev)

        def mat_vjp():
            for lo in range(0, n, ch):
                m = min(ch, n - lo)  # the matrices of this chunk (the last may be shorter)
                ev(kind, alpha, m, A[lo:].data_ptr(), Fm.data_ptr(), Jm.data_ptr(), None, None)
                Abar[lo:lo + m] = torch.einsum("nab,nabcd->ncd", W[lo:lo + m], Jm[:m].view(m, 3, 3, 3, 3))

        def mat_hvp():
            for lo in range(0, n, ch):
                m = min(ch, n - lo)
                ev(kind, alpha, m, A[lo:].data_ptr(), Fm.data_ptr(), Jm.data_ptr(), Hm.data_ptr(), None)
                HV = torch.einsum("nabcdef,ncd->nabef", Hm[:m].view(m, 3, 3, 3, 3, 3, 3), V[lo:lo + m])
                HWV[lo:lo + m] = torch.einsum("nab,nabef->nef", W[lo:lo + m], HV)
                JV[lo:lo + m] = torch.einsum("nabcd,ncd->nab", Jm[:m].view(m, 3, 3, 3, 3), V[lo:lo + m])

        t_mvjp, t_mhvp = timeit(mat_vjp, 1), timeit(mat_hvp, 1)
        del Fm, Jm, Hm
        # FP32: the mixed-precision adjoint kernels on the same values rounded to FP32
        A32, W32, V32 = A.float(), W.float(), V.float()
        Ab32, JV32, HWV32 = torch.empty_like(A32), torch.empty_like(A32), torch.empty_like(A32)
        fn32 = lib.smf_cuda_adjoint_f32 if fam == "smf" else lib.gmf_cuda_adjoint_f32
        vjp32 = lambda: fn32(kind, alpha, n, A32.data_ptr(), W32.data_ptr(), None, None, Ab32.data_ptr(), None, None,
                             None)
        hvp32 = lambda: fn32(kind, alpha, n, A32.data_ptr(), W32.data_ptr(), V32.data_ptr(), None, None,
                             JV32.data_ptr(), HWV32.data_ptr(), None)
        t_vjp32, t_hvp32 = timeit(vjp32), timeit(hvp32)
        # errors of the FP32 results against the FP64 adjoints on the FP32-rounded values (a sample)
        m = min(n, 1 << 16)
        ref = {k: torch.empty((m, 3, 3), dtype=torch.float64, device=dev) for k in ("Abar", "JV", "HWV")}
        A64s, W64s, V64s = A32[:m].double(), W32[:m].double(), V32[:m].double()  # kept alive over the launch
        assert fn(kind, alpha, m, A64s.data_ptr(), W64s.data_ptr(), V64s.data_ptr(), None, ref["Abar"].data_ptr(),
                  ref["JV"].data_ptr(), ref["HWV"].data_ptr(), None) == 0
        assert vjp32() == 0
        torch.cuda.synchronize()
        err = {}
        for k, got in (("Abar", Ab32), ("JV", JV32), ("HWV", HWV32)):
            a, b = got[:m].double(), ref[k]
            ok = ~(torch.isnan(a) & torch.isnan(b))
            err[k] = float((a - b)[ok].abs().max() / b[ok].abs().max())
        res[f"{fam}_{'log' if kind == 1 else 'pow0.3'}"] = {
            "n": n, "vjp_matrices_per_s": n / (t_vjp * 1e-3), "hvp_matrices_per_s": n / (t_hvp * 1e-3),
            "materialised_vjp_matrices_per_s": n / (t_mvjp * 1e-3),
            "materialised_hvp_matrices_per_s": n / (t_mhvp * 1e-3),
            "vjp_speedup": t_mvjp / t_vjp, "hvp_speedup": t_mhvp / t_hvp,
            "f32": {"vjp_matrices_per_s": n / (t_vjp32 * 1e-3), "hvp_matrices_per_s": n / (t_hvp32 * 1e-3),
                    "vjp_speedup_vs_fp64_adjoint": t_vjp / t_vjp32, "hvp_speedup_vs_fp64_adjoint": t_hvp / t_hvp32,
                    "max_rel_err_vs_fp64": err, "err_sample": m},
            "bytes_per_matrix": {"vjp": 216, "hvp": 288}}
    return res


def batched_c3(lib, args, dev):
    """C3: 64 requests, sizes log-uniform in [1e3, 1e6] rescaled to ~8e6 matrices in total, each with a random kind,
    order in {0, 1, 2}, family in {smf Voigt, smf matrix, gmf} and precision (FP32 for smf only), inputs from the C0 /
    C1 generators: one autotuned persistent launch replayed from a CUDA graph, against the 64 single-entry launches"""
    import torch

    from matfun_gb300 import autotune, batched
    from matfun_gb300 import workloads as w
    rng = np.random.default_rng(3)
    sizes = 10.0 ** rng.uniform(3.0, 6.0, 64)
    sizes = np.maximum(1000, (sizes * args.c3_total / sizes.sum()).astype(np.int64))
    pool_s = w.c0_smf_spd(int(sizes.max()), seed=7, as_voigt=False)
    pool_g = w.c1_gmf_groups(int(sizes.max()), seed=8)
    reqs = []
    for i, n in enumerate(sizes):
        fam = ["smf_voigt", "smf", "gmf"][rng.integers(3)]
        kind = ["exp", "log", "sqrt", "pow"][rng.integers(4)]
        order = int(rng.integers(3))
        f32 = fam != "gmf" and rng.uniform() < 0.5
        src = pool_g[:n] if fam == "gmf" else pool_s[:n]
        if fam == "smf_voigt":
            src = w.voigt(src)
        t = torch.from_numpy(np.ascontiguousarray(src)).to(dev)
        reqs.append(batched.request(fam, kind, t.float() if f32 else t, order=order,
                                    alpha=float(rng.uniform(0.1, 0.9)) if kind == "pow" else None))
    total = int(sum(r.n for r in reqs))
    choice, tune_ms = autotune.tune(reqs, reps=1, save=False)
    plan = batched.Plan(reqs)
    st = torch.cuda.Stream(dev)
    st.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(st):
        plan.run()
    torch.cuda.current_stream(dev).wait_stream(st)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()
    fns = {(0, 0): lib.smf_cuda_eval, (1, 0): lib.smf_cuda_eval_matrix, (2, 0): lib.gmf_cuda_eval,
           (0, 1): lib.smf_cuda_eval_f32, (1, 1): lib.smf_cuda_eval_matrix_f32}
    p = lambda t: None if t is None else t.data_ptr()

    def singles():
        for r in reqs:
            c = r.c
            fns[(c.family, c.dtype)](c.kind, c.alpha, c.n, r.x.data_ptr(), p(r.F), p(r.J), p(r.H), None)

    def timeit(f, reps):
        f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            f()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    t_graph = timeit(g.replay, args.c3_steps)
    t_single = timeit(singles, args.c3_steps)
    return {"workload": "64 requests, sizes log-uniform [1e3,1e6], mixed family/kind/order/precision (C3)",
            "matrices": total, "requests": len(reqs),
            "batched_graph_matrices_per_s": total / (t_graph * 1e-3), "batched_ms": t_graph,
            "single_launches_matrices_per_s": total / (t_single * 1e-3), "single_ms": t_single,
            "speedup": t_single / t_graph, "autotuned": choice,
            "autotune_ms": {k: round(v, 3) for k, v in tune_ms.items()}}


def run_ours(args, rank, world, local):
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    lib = matfun_gb300.load()
    kind = KINDS[args.kind]
    n = args.n
    X = w.c1_gmf_groups(n, seed=rank_seed(rank)).reshape(n, 9)
    dev = torch.device("cuda", local)
    dA = torch.from_numpy(X).to(dev)
    dF = torch.empty((n, 9), dtype=torch.float64, device=dev)
    dJ = torch.empty((n, 81), dtype=torch.float64, device=dev)
    dH = torch.empty((n, 729), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream

    def step():
        r = lib.gmf_cuda_eval(kind, args.alpha, n, dA.data_ptr(), dF.data_ptr(), dJ.data_ptr(), dH.data_ptr(), sp)
        if r != 0:
            raise RuntimeError(f"gmf_cuda_eval returned {r}")

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        ev1.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(ms, world)
    value = whole_job_rate(n, ms, world)

    # e2e: the host-buffer C ABI (gmf_cuda_eval_host: the reference's gmf_eval signature on host arrays) on
    # page-locked host arrays: the kernels read A and write F, J, H in host memory over the host link, inside the
    # timed region
    hA = torch.from_numpy(X).pin_memory()
    hF = torch.empty((n, 9), dtype=torch.float64).pin_memory()
    hJ = torch.empty((n, 81), dtype=torch.float64).pin_memory()
    hH = torch.empty((n, 729), dtype=torch.float64).pin_memory()

    def e2e_step():
        r = lib.gmf_cuda_eval_host(kind, args.alpha, n, hA.data_ptr(), hF.data_ptr(), hJ.data_ptr(), hH.data_ptr())
        if r != 0:
            raise RuntimeError(f"gmf_cuda_eval_host returned {r}")

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier(world)
    e2e_steps = max(2, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()  # synchronous: returns when the results are in host memory
    e2e_ms = max_over_ranks(1e3 * (time.perf_counter() - t0) / e2e_steps, world)
    e2e_value = whole_job_rate(n, e2e_ms, world)
    # result check of the last e2e step against the device result: the host path evaluates the batch in its given
    # order, the device path ordered by spectral class, so a matrix may take the real or the complex form of the
    # series depending on its warp neighbours (last-bit differences)
    for h, d in ((hH[:4], dH[:4]), (hF[-4:], dF[-4:])):
        d = d.cpu()
        assert torch.equal(torch.isnan(h), torch.isnan(d))
        ok = ~torch.isnan(d)
        if ok.any():
            assert (h - d).abs()[ok].max() <= 1e-13 * d.abs()[ok].max()

    hbm, peak_kind = peaks()
    import ctypes
    fp64_peak = ctypes.c_double(0.0)
    fp64_ok = lib.matfun_cuda_fp64_peak(ctypes.byref(fp64_peak)) == 0
    achieved = BYTES_PER_MATRIX[2] * n / (ms * 1e-3) / 1e9
    out = None
    if rank == 0:
        out = {"metric": METRIC.replace("log", args.kind), "value": value, "unit": "matrices/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": f"gmf {args.kind} order 2 (F, J, H), general 3x3 FP64, four equal groups: "
                                      "I+0.3N / rotation x stretch / shear / shear x (1+1e-10 N), seed 1+rank",
                          "n_per_gpu": n, "bytes_per_matrix": BYTES_PER_MATRIX[2],
                          "l2": "no flush: 6.9 GB of traffic per step >> 126 MB L2",
                          "parallelism": f"independent matrices x{world}"},
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                            "frac": achieved / hbm, "peak_source": peak_kind,
                            "traffic": (NCU_DRAM_BYTES_PER_MATRIX * n / 1e9) if args.kind == "log" else None,
                            "traffic_unit": "GB per launch",
                            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the ordered "
                                              "gmf_kernel<LOG,2> launch at n=262144 (1853.5 MB), scaled by n",
                            "note": "algorithmic bytes (72 in + 6552 out per matrix) / event time; the kernel is "
                                    "bound by the FP64 pipe (see fp64), not by HBM"},
               "fp64": {"peak_tflops": fp64_peak.value if fp64_ok else None,
                        "peak_source": "measured live: 8 independent DFMA chains per thread (matfun_cuda_fp64_peak)",
                        "achieved_tflops": FP64_FLOP_PER_MATRIX.get(args.kind, 0) * n / (ms * 1e-3) / 1e12 or None,
                        "flop_per_matrix": FP64_FLOP_PER_MATRIX.get(args.kind),
                        "flop_source": "ncu dfma x2 + dadd + dmul per matrix, gmf_kernel<LOG,2> + gmf_key_kernel, "
                                       "this workload"},
               "e2e": {"value": e2e_value, "unit": "matrices/s", "h2d_bytes_per_step": int(hA.numel() * 8),
                       "d2h_bytes_per_step": int((hF.numel() + hJ.numel() + hH.numel()) * 8),
                       "ms_per_step": e2e_ms, "api": "gmf_cuda_eval_host",
                       "timer": "host wall clock around the synchronous call"},
               "gpu_launches": args.steps * launches_per_call(args.kind, n),
               "clocks": clk.summary()}
    del dA, dF, dJ, dH
    if rank == 0 and not args.no_mixed:
        section(out, "mixed", lambda: mixed_vs_fp64(lib, args, dev, hbm))
        section(out, "mixed_gmf", lambda: mixed_gmf_vs_fp64(lib, args, dev, hbm))
    if rank == 0:
        section(out, "smf_c0", lambda: smf_c0(lib, args, dev))
    if rank == 0 and args.mixed_sweep:
        section(out, "mixed_sweep", lambda: mixed_sweep(lib, args, dev, hbm))
    if rank == 0 and not args.no_adjoint:
        section(out, "adjoint", lambda: adjoint_vs_materialised(lib, args, dev))
        section(out, "tangent", lambda: tangent_vs_materialised(lib, args, dev))
    if rank == 0 and not args.no_batched:
        section(out, "batched", lambda: batched_c3(lib, args, dev))
    if rank == 0 and not args.no_cpu:
        Xs = np.ascontiguousarray(X[np.concatenate([np.arange(g * n // 4, g * n // 4 + args.cpu_sample // 4)
                                                    for g in range(4)])])
        rate, cores, kind_s, done = cpu_rate(kind, args.alpha, Xs, 2, budget_s=args.cpu_budget)
        out["cpu_baseline"] = {"value": rate, "unit": "matrices/s", "cores": cores, "kind": kind_s,
                               "sample": f"{done} matrices in repeated calls of {len(Xs)} (equal parts of the four "
                                         f"groups) over >= {args.cpu_budget:.0f} s, OpenMP on all host threads"}
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kind", default="log", choices=["exp", "log", "sqrt"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--cpu-sample", type=int, default=1 << 14)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--c3-total", type=int, default=8_000_000)
    ap.add_argument("--c3-steps", type=int, default=3)
    ap.add_argument("--adj-n", type=int, default=1 << 22)
    ap.add_argument("--mixed-n", type=int, default=1 << 24)
    ap.add_argument("--mixed-steps", type=int, default=5)
    ap.add_argument("--gmf-mixed-n", type=int, default=1 << 20)
    ap.add_argument("--mixed-sweep", action="store_true", help="also the C2 workload over every kind and order")
    ap.add_argument("--smf-n", type=int, default=1 << 16, help="matrices of the C0 section (smf log order 2)")
    args = ap.parse_args()
    args.alpha = 0.5 if args.kind == "sqrt" else 0.0
    if args.kind == "sqrt":
        args.alpha = 0.0  # sqrt ignores alpha (mapped to pow 0.5 inside)
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, rank, world)
        return
    rank, world, local = dist_setup(args.gpus)
    run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Benchmark: gmf log, order 2 (F, J, H), FP64, n = 2^20 general 3x3 matrices in the four groups of the reference's
workload (real spectra, rotations with stretch, shears, near-confluent shears), through the C ABI of
libmatfun_cuda (gmf_cuda_eval); then every other configuration of the same path, each with its rooflines and the CPU
implementation timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--kind log] [--n 1048576]
    python bench.py --count-pass        (one small launch per configuration, for the ncu instruction counts)

One JSON line on rank 0.  `value` is whole-job matrices/s with inputs resident in HBM (CUDA events on the launching
stream; the per-step traffic of 6.9 GB is far above the 126 MB L2, so no flush is needed); `e2e` is the same metric
through the host-buffer C ABI (gmf_cuda_eval_host, the reference's gmf_eval signature on host arrays) from page-locked
HOST arrays, with all host-device copies inside the timed region (host wall clock around the synchronous call).
`roofline` names the binding bound of the headline kernel (the FP64 pipe) and carries the HBM fraction beside it.

Sections (each with `roofline` and `cpu_baseline`): c1_kinds (exp, sqrt of the headline workload), smf_c0 (smf log
order 2, Voigt, n = 65536), mixed (smf FP32 storage against FP64 over every kind and order, n = 2^24, with errors per
batch and per matrix), mixed_gmf (gmf FP32 storage against FP64, every kind, order 2), batched (64 mixed requests in
one persistent launch), adjoint (VJP / HVP without J or H, FP64 and FP32), tangent (|log A|^2 / 2: F, J^T F,
J^T J + F : H fused).

Multi-GPU (torchrun): every rank evaluates its own n matrices (independent matrices, no collective on the data path).
--impl reference times the CPU implementation of the same path on the host cores (the reference's compiled library
where it was built, otherwise the oracle restatement of it) on the same workload.
"""
import argparse
import ctypes
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
METRIC = "gmf log order-2 matrices/s (FP64)"


def io_bytes(fam, order, elem=8):
    """algorithmic bytes per matrix of one evaluation: the input and the outputs F (+ J) (+ H), each read or written
    once (fam: "smf_voigt" 6 entries per matrix, "smf" / "gmf" 9)"""
    nf = 6 if fam == "smf_voigt" else 9
    return elem * (nf + sum(nf ** (k + 1) for k in range(order + 1)))


# Executed floating-point operations per matrix (2 per FMA, 1 per add or multiply; FP64 pipe: DFMA, DADD, DMUL; FP32
# pipe: FFMA, FADD, FMUL) of each configuration's kernels, from the ncu counters
# smsp__sass_thread_inst_executed_op_{d,f}{fma,add,mul}_pred_on.sum of `python bench.py --count-pass` divided by the
# matrices of each launch (profiles/pipe_counts_all_configs.md).  They turn the measured time of a configuration into
# its FP64 / FP32 pipe fraction.  None: the kernels execute no instruction of that pipe.
PIPE_FLOPS = {
    "gmf/log/2/f64": {"fp64": 5438, "fp32": 7486},
    "gmf/exp/2/f64": {"fp64": 4912, "fp32": 6229},
    "gmf/sqrt/2/f64": {"fp64": 7873, "fp32": 12200},
    "gmf/log/2/f32": {"fp64": 1687, "fp32": 20409},
    "gmf/exp/2/f32": {"fp64": 2641, "fp32": 9646},
    "gmf/sqrt/2/f32": {"fp64": 3804, "fp32": 20265},
    "gmf/pow0.3/2/f32": {"fp64": 4468, "fp32": 20323},
    "gmf/log/tangent/f64": {"fp64": 7661, "fp32": 7534},
    "smf/log/2/f64/c0": {"fp64": 2577, "fp32": 45},
    "smf/exp/0/f32": {"fp64": None, "fp32": 1931},
    "smf/exp/0/f64": {"fp64": 701, "fp32": 14},
    "smf/exp/1/f32": {"fp64": None, "fp32": 2330},
    "smf/exp/1/f64": {"fp64": 1104, "fp32": 20},
    "smf/exp/2/f32": {"fp64": None, "fp32": 3463},
    "smf/exp/2/f64": {"fp64": 2348, "fp32": 214},
    "smf/log/0/f32": {"fp64": None, "fp32": 2189},
    "smf/log/0/f64": {"fp64": 882, "fp32": 22},
    "smf/log/1/f32": {"fp64": None, "fp32": 2629},
    "smf/log/1/f64": {"fp64": 1290, "fp32": 26},
    "smf/log/2/f32": {"fp64": None, "fp32": 3673},
    "smf/log/2/f64": {"fp64": 2664, "fp32": 221},
    "smf/sqrt/0/f32": {"fp64": None, "fp32": 1919},
    "smf/sqrt/0/f64": {"fp64": 653, "fp32": 14},
    "smf/sqrt/1/f32": {"fp64": None, "fp32": 2210},
    "smf/sqrt/1/f64": {"fp64": 999, "fp32": 14},
    "smf/sqrt/2/f32": {"fp64": None, "fp32": 3284},
    "smf/sqrt/2/f64": {"fp64": 2400, "fp32": 214},
    "smf/pow/0/f32": {"fp64": None, "fp32": 2078},
    "smf/pow/0/f64": {"fp64": 981, "fp32": 14},
    "smf/pow/1/f32": {"fp64": None, "fp32": 2570},
    "smf/pow/1/f64": {"fp64": 1971, "fp32": 19},
    "smf/pow/2/f32": {"fp64": None, "fp32": 3702},
    "smf/pow/2/f64": {"fp64": 3373, "fp32": 219},
    "smf/log/vjp/f64": {"fp64": 1320, "fp32": 32},
    "smf/log/hvp/f64": {"fp64": 1870, "fp32": 45},
    "smf/log/vjp/f32": {"fp64": None, "fp32": 2636},
    "smf/log/hvp/f32": {"fp64": None, "fp32": 2992},
    "gmf/pow0.3/vjp/f64": {"fp64": 4288, "fp32": 10652},
    "gmf/pow0.3/hvp/f64": {"fp64": 9067, "fp32": 24339},
    "gmf/pow0.3/vjp/f32": {"fp64": 3263, "fp32": 11624},
    "gmf/pow0.3/hvp/f32": {"fp64": 4874, "fp32": 29369},
}


def pipe_flops(tag):
    return PIPE_FLOPS.get(tag) or {}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class Peaks:
    """the roofline denominators: HBM copy bandwidth (MEASURED_PEAKS.json), and the FP64 / FP32 FMA throughput
    measured live on this GPU (matfun_cuda_fp64_peak / matfun_cuda_fp32_peak)"""

    def __init__(self, lib):
        self.hbm, self.hbm_source = hbm_peak()
        self.fp64 = self.fp32 = None
        v = ctypes.c_double(0.0)
        if lib.matfun_cuda_fp64_peak(ctypes.byref(v)) == 0:
            self.fp64 = v.value
        if lib.matfun_cuda_fp32_peak(ctypes.byref(v)) == 0:
            self.fp32 = v.value


def roofline(n, ms, bytes_per_matrix, tag, pk):
    """the rooflines of one timed configuration: HBM (algorithmic bytes / time) and, where its executed flops per
    matrix are known, the FP64 and FP32 pipes; `bound` names the largest fraction (the binding one), whose figures
    are the top-level achieved / peak / frac, the others are nested under their names"""
    t = ms * 1e-3
    parts = {}
    a = bytes_per_matrix * n / t / 1e9
    parts["hbm"] = {"achieved": a, "peak": pk.hbm, "unit": "GB/s", "frac": a / pk.hbm, "peak_source": pk.hbm_source,
                    "bytes_per_matrix": bytes_per_matrix}
    fl = pipe_flops(tag)
    for pipe, peak in (("fp64", pk.fp64), ("fp32", pk.fp32)):
        if fl.get(pipe) and peak:
            a = fl[pipe] * n / t / 1e12
            parts[pipe] = {"achieved": a, "peak": peak, "unit": "TFLOP/s", "frac": a / peak,
                           "peak_source": f"measured live ({pipe.upper()} FMA chains, matfun_cuda_{pipe}_peak)",
                           "flop_per_matrix": fl[pipe]}
    bound = max(parts, key=lambda k: parts[k]["frac"])
    out = {"bound": bound}
    out.update(parts[bound])
    for k, v in parts.items():
        if k != bound:
            out[k] = v
    if not fl:
        out["pipes"] = "not counted for this configuration"
    return out


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


# ------------------------------------------------------------------------------------------------ CPU implementation
def cpu_lib():
    """(library, kind): the reference's compiled CPU library where it was built, else the oracle restatement"""
    from tests import oracle_lib as ol
    ref = ol.reference()
    return (ref, "reference") if ref is not None else (ol.oracle(), "port")


def cpu_cores():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


class CpuCall:
    """one CPU entry point (smf_eval / smf_eval_matrix / gmf_eval) on fixed host arrays: outputs allocated and touched
    once, so that repeated calls time the evaluation, not page faults"""

    def __init__(self, fam, kind, alpha, X, order):
        self.lib, self.kind_s = cpu_lib()
        self.fn = self.lib[fam]
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        n, nf = len(self.X), self.X.shape[1]
        self.out = [np.zeros((n, nf ** (k + 1))) for k in range(order + 1)] + [None] * (2 - order)
        self.args = (kind, float(alpha), n, self.X.ctypes.data) + tuple(
            None if o is None else o.ctypes.data for o in self.out)

    def __call__(self):
        r = self.fn(*self.args)
        if r not in (0, -3):
            raise RuntimeError(f"CPU call returned {r}")
        return self.out


def cpu_rate(call, budget_s, extra=None):
    """matrices/s of repeated CPU calls (plus `extra(outputs)`, a contraction the configuration adds) until budget_s
    has elapsed, after one untimed call"""
    o = call()
    if extra:
        extra(o)
    done, t0 = 0, time.perf_counter()
    while True:
        o = call()
        if extra:
            extra(o)
        done += len(call.X)
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    return done / el, done, el


def cpu_baseline(call, budget_s, what, extra=None):
    rate, done, el = cpu_rate(call, budget_s, extra)
    return {"value": rate, "unit": "matrices/s", "cores": cpu_cores(), "kind": call.kind_s,
            "sample": f"{what}: {done} matrices in repeated calls of {len(call.X)} over {el:.1f} s, OpenMP on all "
                      f"host threads"}


def group_sample(X, m):
    """m matrices in equal parts from the four groups of the C1 workload"""
    n = len(X)
    return np.ascontiguousarray(np.concatenate([X[g * n // 4: g * n // 4 + m // 4] for g in range(4)]))


def run_reference(args, rank, world):
    """--impl reference: the CPU path on this host's cores, rank 0 only, on the same workload as the headline (all
    n = 2^20 matrices per step)"""
    if rank != 0:
        return
    from matfun_gb300 import workloads as w
    X = w.c1_gmf_groups(args.n, seed=1).reshape(-1, 9)
    call = CpuCall("gmf_eval", KINDS[args.kind], args.alpha, X, 2)
    for _ in range(args.warmup):
        CpuCall("gmf_eval", KINDS[args.kind], args.alpha, X[:4096], 2)()
    call()  # outputs touched
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call()
    el = time.perf_counter() - t0
    rate = args.steps * len(X) / el
    cores = cpu_cores()
    out = {"metric": METRIC.replace("log", args.kind), "value": rate, "unit": "matrices/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": f"gmf {args.kind} order 2 (F, J, H), general 3x3 FP64, four equal groups: "
                                  "I+0.3N / rotation x stretch / shear / shear x (1+1e-10 N), seed 1",
                      "n_per_gpu": args.n},
           "cpu_baseline": {"value": rate, "unit": "matrices/s", "cores": cores, "kind": call.kind_s,
                            "sample": f"the whole workload ({len(X)} matrices) per step, OpenMP on {cores} threads"},
           "e2e": {"value": rate, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------------------------------ GPU helpers
def timed_ms(fn, steps, warmup=2, stream=None):
    """ms per call of fn on the GPU: CUDA events on `stream` (default: the current stream) around `steps` calls,
    after `warmup` untimed calls"""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def err_stats(got, ref):
    """errors of FP32 results against FP64 results on the same input values, (m, k) tensors: per batch (max |x - ref|
    / max |ref| over the array) and per matrix (the same within each row), the per-matrix figure over the rows whose
    largest reference entry lies within FP32's normal range; NaN positions compared"""
    import torch
    a, b = got.double(), ref
    nan_a, nan_b = torch.isnan(a), torch.isnan(b)
    d = torch.where(nan_a & nan_b, torch.zeros_like(a), (a - b).abs())
    d = torch.nan_to_num(d, nan=float("inf"))
    s = torch.nan_to_num(b, nan=0.0).abs()
    smax = s.max(dim=1).values
    rows = d.max(dim=1).values / smax.clamp_min(1e-300)
    fits = (smax <= 3.4028234663852886e38) & (smax >= 1.1754943508222875e-38)
    nan_rows = nan_b.all(dim=1)  # matrices outside the domain: NaN in both
    rf = rows[fits]
    return {"batch": float(d.max() / s.max().clamp_min(1e-300)),
            "per_matrix_max": float(rf.max()) if rf.numel() else None,
            "per_matrix_p99_99": float(torch.quantile(rf[:1 << 20].float(), 0.9999)) if rf.numel() else None,
            "nan_rows": int(nan_rows.sum()), "rows_outside_fp32_range": int((~fits & ~nan_rows).sum()),
            "nan_mismatch_rows": int((nan_a != nan_b).any(1).sum())}


def pair_f32_f64(fn32, fn64, x32, nf, kind, alpha, order, steps, dev, sample=65536):
    """time the FP32 entry point and the FP64 one on the same values; errors of the FP32 results against the FP64
    results on a sample of rows spread over the batch"""
    import torch
    n = x32.shape[0]
    d32 = x32.to(dev)
    d64 = d32.double()
    res = {}
    idx = torch.arange(0, n, max(1, n // sample), device=dev)
    for tag, dt, x, fn in (("f32", torch.float32, d32, fn32), ("f64", torch.float64, d64, fn64)):
        outs = [torch.empty((n, nf ** (k + 1)), dtype=dt, device=dev) for k in range(order + 1)]
        p = [t.data_ptr() for t in outs] + [None] * (2 - order)

        def call():
            r = fn(kind, alpha, n, x.data_ptr(), *p, None)
            if r != 0:
                raise RuntimeError(f"returned {r}")
        ms = timed_ms(call, steps)
        res[tag] = (ms, [t[idx] for t in outs])
        del outs
    err = {name: err_stats(g, r) for name, g, r in zip("FJH", res["f32"][1], res["f64"][1])}
    return res["f32"][0], res["f64"][0], err, int(idx.numel())


# ------------------------------------------------------------------------------------------------ sections
def c1_kinds(lib, args, dev, pk, X):
    """exp and sqrt, order 2, on the headline workload (C1 gmf, FP64, n = 2^20)"""
    import torch
    n = len(X)
    A = torch.from_numpy(X).to(dev)
    F, J, H = (torch.empty((n, k), dtype=torch.float64, device=dev) for k in (9, 81, 729))
    rows = {}
    for name in ("exp", "sqrt"):
        k = KINDS[name]
        ms = timed_ms(lambda: lib.gmf_cuda_eval(k, 0.0, n, A.data_ptr(), F.data_ptr(), J.data_ptr(), H.data_ptr(),
                                                None), max(5, args.steps // 2))
        rows[name] = {"ms": ms, "matrices_per_s": n / (ms * 1e-3),
                      "roofline": roofline(n, ms, io_bytes("gmf", 2), f"gmf/{name}/2/f64", pk),
                      "cpu_baseline": cpu_baseline(CpuCall("gmf_eval", k, 0.0, group_sample(X, 8192), 2),
                                                   args.cpu_budget_section, f"gmf_eval {name} order 2 on the C1 groups")}
    return {"workload": f"C1: gmf exp / sqrt order 2 (F, J, H), n={n} FP64, the four groups", **rows}


def smf_c0(lib, args, dev, pk):
    """C0: smf log order 2 on Voigt vectors, FP64 (n = 65536 SPD matrices with 10 % repeated and 2 % triple
    eigenvalues), through smf_cuda_eval"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.smf_n
    Vh = w.c0_smf_spd(n)
    V = torch.from_numpy(Vh).to(dev)
    F, J, H = (torch.empty((n, k), dtype=torch.float64, device=dev) for k in (6, 36, 216))
    ms = timed_ms(lambda: lib.smf_cuda_eval(1, 0.0, n, V.data_ptr(), F.data_ptr(), J.data_ptr(), H.data_ptr(), None),
                  max(args.steps, 20), 3)
    return {"workload": f"C0: smf log order 2, Voigt, n={n} SPD (10 % repeated, 2 % triple eigenvalues), FP64",
            "ms": ms, "matrices_per_s": n / (ms * 1e-3), "l2": "inputs and outputs 138 MB per call, about the L2 size",
            "roofline": roofline(n, ms, io_bytes("smf_voigt", 2), "smf/log/2/f64/c0", pk),
            "cpu_baseline": cpu_baseline(CpuCall("smf_eval", 1, 0.0, Vh[:16384], 2), args.cpu_budget_section,
                                         "smf_eval log order 2 on C0 matrices")}


def mixed_sweep(lib, args, dev, pk):
    """C2 over every kind and order: smf Voigt, n = 2^24 SPD (condition number log-uniform in [1, 1e6], smallest
    eigenvalue gap log-uniform in [1e-12, 1]) stored as FP32; pow with one exponent alpha ~ U(0.1, 0.9) per call,
    seeded.  The mixed-precision path against the FP64 path on the same values, with the errors of the FP32 results
    per batch and per matrix"""
    import torch

    from matfun_gb300 import autotune
    from matfun_gb300 import workloads as w
    n = args.mixed_n
    xh = w.c2_smf_spd(n, seed=2)
    x32 = torch.from_numpy(xh)
    xd = x32.to(dev)
    path, path_ms = autotune.tune_smf_f32(xd, save=False)  # the store path of orders 1 and 2, timed on log
    del xd
    rng = np.random.default_rng(2)
    rows = []
    for name, kind in (("exp", 0), ("log", 1), ("sqrt", 3), ("pow", 2)):
        alpha = float(rng.uniform(0.1, 0.9)) if kind == 2 else 0.0
        for order in (0, 1, 2):
            ms32, ms64, err, ns = pair_f32_f64(lib.smf_cuda_eval_f32, lib.smf_cuda_eval, x32, 6, kind, alpha, order,
                                               args.mixed_steps, dev)
            call = CpuCall("smf_eval", kind, alpha, xh[:16384].astype(np.float64), order)
            rf32 = roofline(n, ms32, io_bytes("smf_voigt", order, 4), f"smf/{name}/{order}/f32", pk)
            rows.append({"kind": name, "alpha": alpha, "order": order, "mixed_ms": ms32, "fp64_ms": ms64,
                         "mixed_matrices_per_s": n / (ms32 * 1e-3), "fp64_matrices_per_s": n / (ms64 * 1e-3),
                         "speedup_vs_fp64": ms64 / ms32, "err_vs_fp64": err,
                         "mixed_hbm_frac": rf32["hbm"]["frac"] if "hbm" in rf32 else rf32["frac"],
                         "roofline": rf32,
                         "fp64_roofline": roofline(n, ms64, io_bytes("smf_voigt", order), f"smf/{name}/{order}/f64",
                                                   pk),
                         "cpu_baseline": cpu_baseline(call, args.cpu_budget_row,
                                                      f"smf_eval {name} order {order} (FP64) on C2 matrices")})
            torch.cuda.empty_cache()
    return {"workload": f"C2: smf Voigt, n={n} SPD, condition log-uniform [1,1e6], smallest gap log-uniform "
                        "[1e-12,1], FP32 storage; every kind and order; errors of the FP32 results against the FP64 "
                        "path on the same values (per batch, and per matrix where its outputs fit FP32's range)",
            "err_sample": ns, "rows": rows,
            "log_o2_mixed_hbm_frac": next(r["mixed_hbm_frac"] for r in rows if r["kind"] == "log" and r["order"] == 2),
            "store_path": {"chosen": {str(o): autotune.SMF_F32_PATHS[p] for o, p in path.items()},
                           "log_ms": {str(o): {autotune.SMF_F32_PATHS[p]: round(t, 4) for p, t in d.items()}
                                      for o, d in path_ms.items()}}}


def mixed_gmf(lib, args, dev, pk, cpu_log):
    """gmf at order 2 on the C1 workload (n = 2^20, the four groups) stored as FP32: the mixed-precision gmf path
    against the FP64 path on the same values, every kind"""
    from matfun_gb300 import workloads as w
    import torch
    n = args.gmf_mixed_n
    xh = w.c1_gmf_groups(n, seed=1).astype(np.float32).reshape(n, 9)
    x32 = torch.from_numpy(xh)
    rows = {}
    for name, kind, alpha in (("log", 1, 0.0), ("exp", 0, 0.0), ("sqrt", 3, 0.0), ("pow0.3", 2, 0.3)):
        ms32, ms64, err, ns = pair_f32_f64(lib.gmf_cuda_eval_f32, lib.gmf_cuda_eval, x32, 9, kind, alpha, 2,
                                           args.mixed_steps, dev)
        if name == "log" and cpu_log is not None:
            cb = cpu_log
        else:
            cb = cpu_baseline(CpuCall("gmf_eval", kind, alpha, group_sample(xh.astype(np.float64), 4096), 2),
                              args.cpu_budget_row, f"gmf_eval {name} order 2 (FP64) on the C1 groups")
        rows[name] = {"mixed_ms": ms32, "fp64_ms": ms64, "mixed_matrices_per_s": n / (ms32 * 1e-3),
                      "fp64_matrices_per_s": n / (ms64 * 1e-3), "speedup_vs_fp64": ms64 / ms32, "err_vs_fp64": err,
                      "roofline": roofline(n, ms32, io_bytes("gmf", 2, 4), f"gmf/{name}/2/f32", pk),
                      "cpu_baseline": cb}
    return {"workload": f"gmf order 2, n={n} general matrices (C1 groups), FP32 storage, against the FP64 path on the "
                        "same values", "err_sample": ns, **rows}


def tangent_vs_materialised(lib, args, dev, pk, X):
    """the tangent of psi(A) = |log A|^2 / 2 (G = J^T F, K = J^T J + F : H) on the C1 workload, n = 2^20 FP64: the
    fused kernel (gmf_cuda_tangent, no J or H formed) against evaluating F, J, H (gmf_cuda_eval) and contracting them
    with torch (bmm), with the max relative difference of the two on the whole batch"""
    import torch
    n = len(X)
    A = torch.from_numpy(X).to(dev)
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

    t_f = timed_ms(fused, 3)
    t_u = timed_ms(unfused, 3)
    Gu, Ku = unfused()
    torch.cuda.synchronize()

    def rel(a, b):
        d = torch.where(torch.isnan(a) & torch.isnan(b), torch.zeros_like(a), (a - b).abs())
        return float(d.max() / torch.nan_to_num(b, nan=0.0).abs().max())

    def contract(o):  # the same contraction on the CPU outputs
        Fo, Jo, Ho = o[0], o[1].reshape(-1, 9, 9), o[2].reshape(-1, 9, 81)
        np.einsum("nab,nbc->nac", Fo[:, None, :], Jo)
        np.einsum("nba,nbc->nac", Jo, Jo) + np.einsum("na,nab->nb", Fo, Ho).reshape(-1, 9, 9)

    call = CpuCall("gmf_eval", 1, 0.0, group_sample(X, 4096), 2)
    return {"workload": f"psi(A) = |log A|^2 / 2 on C1, n={n} FP64: F, G = J^T F, K = J^T J + F : H",
            "fused_matrices_per_s": n / (t_f * 1e-3), "fused_ms": t_f,
            "materialised_matrices_per_s": n / (t_u * 1e-3), "materialised_ms": t_u, "speedup": t_u / t_f,
            "bytes_written_per_matrix": {"fused": 8 * (9 + 9 + 81), "materialised": 8 * (9 + 81 + 729) + 8 * 90},
            "max_rel_diff_G": rel(G, Gu), "max_rel_diff_K": rel(K, Ku.reshape(n, 81)),
            "roofline": roofline(n, t_f, 8 * (9 + 9 + 9 + 81), "gmf/log/tangent/f64", pk),
            "cpu_baseline": cpu_baseline(call, args.cpu_budget_section,
                                         "gmf_eval log order 2 + the contractions J^T F, J^T J + F : H (numpy)",
                                         contract)}


def adjoint_vs_materialised(lib, args, dev, pk):
    """C4: the gradient of L = sum <W, f(A)> and its Hessian-vector product along V, for smf log (SPD, the C0
    generator) and gmf pow 0.3 (real and rotation groups of C1), n = 2^22, FP64 and FP32: the adjoint kernels (no J,
    H formed) against evaluating J (resp. H) with the eval kernels and contracting it with W (resp. W and V)"""
    import torch

    from matfun_gb300 import workloads as w
    n = args.adj_n
    res = {}
    for fam, kind, alpha in (("smf", 1, 0.0), ("gmf", 2, 0.3)):
        name = "log" if kind == 1 else "pow0.3"
        if fam == "smf":
            Ah = w.c0_smf_spd(n, seed=4, as_voigt=False)
        else:
            Ah = w.c1_gmf_groups(2 * n, seed=4)[: n]
        A = torch.from_numpy(Ah).to(dev)
        g = torch.Generator(device=dev).manual_seed(5)
        W = torch.randn(A.shape, dtype=torch.float64, device=dev, generator=g)
        V = torch.randn(A.shape, dtype=torch.float64, device=dev, generator=g)
        Abar, HWV, JV = torch.empty_like(A), torch.empty_like(A), torch.empty_like(A)
        fn = lib.smf_cuda_adjoint if fam == "smf" else lib.gmf_cuda_adjoint
        ev = lib.smf_cuda_eval_matrix if fam == "smf" else lib.gmf_cuda_eval
        vjp = lambda: fn(kind, alpha, n, A.data_ptr(), W.data_ptr(), None, None, Abar.data_ptr(), None, None, None)
        hvp = lambda: fn(kind, alpha, n, A.data_ptr(), W.data_ptr(), V.data_ptr(), None, None, JV.data_ptr(),
                         HWV.data_ptr(), None)
        t_vjp, t_hvp = timed_ms(vjp, 3, 1), timed_ms(hvp, 3, 1)
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

        t_mvjp, t_mhvp = timed_ms(mat_vjp, 1, 1), timed_ms(mat_hvp, 1, 1)
        del Fm, Jm, Hm
        # FP32: the mixed-precision adjoint kernels on the same values rounded to FP32
        A32, W32, V32 = A.float(), W.float(), V.float()
        Ab32, JV32, HWV32 = torch.empty_like(A32), torch.empty_like(A32), torch.empty_like(A32)
        fn32 = lib.smf_cuda_adjoint_f32 if fam == "smf" else lib.gmf_cuda_adjoint_f32
        vjp32 = lambda: fn32(kind, alpha, n, A32.data_ptr(), W32.data_ptr(), None, None, Ab32.data_ptr(), None, None,
                             None)
        hvp32 = lambda: fn32(kind, alpha, n, A32.data_ptr(), W32.data_ptr(), V32.data_ptr(), None, None,
                             JV32.data_ptr(), HWV32.data_ptr(), None)
        t_vjp32, t_hvp32 = timed_ms(vjp32, 3, 1), timed_ms(hvp32, 3, 1)
        # errors of the FP32 results against the FP64 adjoints on the FP32-rounded values (a sample)
        m = min(n, 1 << 16)
        ref = {k: torch.empty((m, 3, 3), dtype=torch.float64, device=dev) for k in ("Abar", "JV", "HWV")}
        A64s, W64s, V64s = A32[:m].double(), W32[:m].double(), V32[:m].double()  # kept alive over the launch
        assert fn(kind, alpha, m, A64s.data_ptr(), W64s.data_ptr(), V64s.data_ptr(), None, ref["Abar"].data_ptr(),
                  ref["JV"].data_ptr(), ref["HWV"].data_ptr(), None) == 0
        assert vjp32() == 0 and hvp32() == 0
        torch.cuda.synchronize()
        err = {k: err_stats(got[:m].reshape(m, 9), ref[k].reshape(m, 9))
               for k, got in (("Abar", Ab32), ("JV", JV32), ("HWV", HWV32))}
        # the CPU path: the reference's evaluation (order 1 resp. 2) and the same contractions with numpy
        cfam = "smf_eval_matrix" if fam == "smf" else "gmf_eval"
        s = 4096
        Wh, Vh = W[:s].cpu().numpy(), V[:s].cpu().numpy()
        cv = CpuCall(cfam, kind, alpha, Ah[:s].reshape(s, 9), 1)
        ch_ = CpuCall(cfam, kind, alpha, Ah[:s].reshape(s, 9), 2)
        c_vjp = lambda o: np.einsum("nab,nabcd->ncd", Wh, o[1].reshape(s, 3, 3, 3, 3))
        c_hvp = lambda o: (np.einsum("nab,nabef->nef", Wh, np.einsum("nabcdef,ncd->nabef",
                                                                     o[2].reshape(s, 3, 3, 3, 3, 3, 3), Vh)),
                           np.einsum("nabcd,ncd->nab", o[1].reshape(s, 3, 3, 3, 3), Vh))
        res[f"{fam}_{name}"] = {
            "n": n, "vjp_matrices_per_s": n / (t_vjp * 1e-3), "hvp_matrices_per_s": n / (t_hvp * 1e-3),
            "materialised_vjp_matrices_per_s": n / (t_mvjp * 1e-3),
            "materialised_hvp_matrices_per_s": n / (t_mhvp * 1e-3),
            "vjp_speedup": t_mvjp / t_vjp, "hvp_speedup": t_mhvp / t_hvp,
            "roofline": {"vjp": roofline(n, t_vjp, 216, f"{fam}/{name}/vjp/f64", pk),
                         "hvp": roofline(n, t_hvp, 288 + 72, f"{fam}/{name}/hvp/f64", pk)},
            "f32": {"vjp_matrices_per_s": n / (t_vjp32 * 1e-3), "hvp_matrices_per_s": n / (t_hvp32 * 1e-3),
                    "vjp_speedup_vs_fp64_adjoint": t_vjp / t_vjp32, "hvp_speedup_vs_fp64_adjoint": t_hvp / t_hvp32,
                    "err_vs_fp64": err, "err_sample": m,
                    "roofline": {"vjp": roofline(n, t_vjp32, 108, f"{fam}/{name}/vjp/f32", pk),
                                 "hvp": roofline(n, t_hvp32, 180, f"{fam}/{name}/hvp/f32", pk)}},
            "bytes_per_matrix": {"vjp": 216, "hvp": 360, "note": "HVP: A, W, V in, J V and W.H.V out"},
            "cpu_baseline": {"vjp": cpu_baseline(cv, args.cpu_budget_row,
                                                 f"{cfam} {name} order 1 + J^T W (numpy)", c_vjp),
                             "hvp": cpu_baseline(ch_, args.cpu_budget_row,
                                                 f"{cfam} {name} order 2 + W.H.V and J V (numpy)", c_hvp)}}
        del A, W, V, Abar, HWV, JV, A32, W32, V32, Ab32, JV32, HWV32
        torch.cuda.empty_cache()
    return res


def batched_c3(lib, args, dev, pk):
    """C3: 64 requests, sizes log-uniform in [1e3, 1e6] rescaled to ~8e6 matrices in total, each with a random kind,
    order in {0, 1, 2}, family in {smf Voigt, smf matrix, gmf} and precision (FP32 / FP64), inputs from the C0 / C1
    generators: one autotuned persistent launch replayed from a CUDA graph, against the 64 single-entry launches"""
    import torch

    from matfun_gb300 import autotune, batched
    from matfun_gb300 import workloads as w
    rng = np.random.default_rng(3)
    sizes = 10.0 ** rng.uniform(3.0, 6.0, 64)
    sizes = np.maximum(1000, (sizes * args.c3_total / sizes.sum()).astype(np.int64))
    pool_s = w.c0_smf_spd(int(sizes.max()), seed=7, as_voigt=False)
    pool_g = w.c1_gmf_groups(int(sizes.max()), seed=8)
    reqs, meta = [], []
    for i, n in enumerate(sizes):
        fam = ["smf_voigt", "smf", "gmf"][rng.integers(3)]
        kind = ["exp", "log", "sqrt", "pow"][rng.integers(4)]
        order = int(rng.integers(3))
        f32 = rng.uniform() < 0.5
        alpha = float(rng.uniform(0.1, 0.9)) if kind == "pow" else None
        src = pool_g[:n] if fam == "gmf" else pool_s[:n]
        if fam == "smf_voigt":
            src = w.voigt(src)
        src = np.ascontiguousarray(src)
        t = torch.from_numpy(src).to(dev)
        reqs.append(batched.request(fam, kind, t.float() if f32 else t, order=order, alpha=alpha))
        meta.append((fam, kind, order, f32, alpha, src))
    total = int(sum(r.n for r in reqs))
    nbytes = sum(io_bytes(fam, order, 4 if f32 else 8) * r.n for r, (fam, _, order, f32, _, _) in zip(reqs, meta))
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
           (0, 1): lib.smf_cuda_eval_f32, (1, 1): lib.smf_cuda_eval_matrix_f32, (2, 1): lib.gmf_cuda_eval_f32}
    p = lambda t: None if t is None else t.data_ptr()

    def singles(fams=(0, 1, 2)):
        for r in reqs:
            c = r.c
            if c.family in fams:
                fns[(c.family, c.dtype)](c.kind, c.alpha, c.n, r.x.data_ptr(), p(r.F), p(r.J), p(r.H), None)

    t_graph = timed_ms(g.replay, args.c3_steps, 1)
    t_single = timed_ms(singles, args.c3_steps, 1)
    # where the single launches spend their time: the general family's requests alone, the symmetric ones alone
    t_single_gmf = timed_ms(lambda: singles((2,)), args.c3_steps, 1)
    t_single_smf = timed_ms(lambda: singles((0, 1)), args.c3_steps, 1)
    # the CPU path: each request's FP64 entry point on a sample of its inputs, its time scaled to the request's size
    cpu_s, sampled = 0.0, 0
    cfam = {"smf_voigt": "smf_eval", "smf": "smf_eval_matrix", "gmf": "gmf_eval"}
    for r, (fam, kind, order, f32, alpha, src) in zip(reqs, meta):
        s = min(r.n, 2048)
        X = src[:s].reshape(s, -1).astype(np.float64)
        if f32:
            X = X.astype(np.float32).astype(np.float64)
        call = CpuCall(cfam[fam], KINDS[kind], alpha or 0.0, X, order)
        rate, _, _ = cpu_rate(call, 0.02)
        cpu_s += r.n / rate
        sampled += s
    cores = cpu_cores()
    return {"workload": "64 requests, sizes log-uniform [1e3,1e6], mixed family/kind/order/precision (C3)",
            "matrices": total, "requests": len(reqs), "fp32_requests": int(sum(m[3] for m in meta)),
            "gmf_fp32_requests": int(sum(m[3] and m[0] == "gmf" for m in meta)),
            "batched_graph_matrices_per_s": total / (t_graph * 1e-3), "batched_ms": t_graph,
            "single_launches_matrices_per_s": total / (t_single * 1e-3), "single_ms": t_single,
            "speedup": t_single / t_graph, "autotuned": choice,
            "tile_matrices": {"gmf": 128, "smf": int(choice.get("smf_tile", 128))},
            "single_ms_by_family": {"gmf": t_single_gmf, "smf": t_single_smf},
            "gmf_matrices": int(sum(r.n for r, m in zip(reqs, meta) if m[0] == "gmf")),
            "autotune_ms": {k: round(v, 3) for k, v in tune_ms.items()},
            "roofline": roofline(total, t_graph, nbytes / total, "batched/c3", pk),
            "cpu_baseline": {"value": total / cpu_s, "unit": "matrices/s", "cores": cores, "kind": cpu_lib()[1],
                             "sample": f"each request's FP64 CPU entry point timed on up to 2048 of its matrices "
                                       f"({sampled} in all, >= 20 ms per request), scaled to its size; "
                                       f"FP32 requests on their FP32-rounded values"}}


# ------------------------------------------------------------------------------------------------ the headline
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
    del hA, hF, hJ, hH

    pk = Peaks(lib)
    out = None
    if rank == 0:
        rf = roofline(n, ms, io_bytes("gmf", 2), f"gmf/{args.kind}/2/f64", pk)
        rf["traffic"] = (NCU_DRAM_BYTES_PER_MATRIX * n / 1e9) if args.kind == "log" else None
        rf["traffic_unit"] = "GB per launch"
        rf["traffic_source"] = NCU_TRAFFIC_SOURCE
        out = {"metric": METRIC.replace("log", args.kind), "value": value, "unit": "matrices/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": f"gmf {args.kind} order 2 (F, J, H), general 3x3 FP64, four equal groups: "
                                      "I+0.3N / rotation x stretch / shear / shear x (1+1e-10 N), seed 1+rank",
                          "n_per_gpu": n, "bytes_per_matrix": io_bytes("gmf", 2),
                          "l2": "no flush: 6.9 GB of traffic per step >> 126 MB L2",
                          "parallelism": f"independent matrices x{world}"},
               "roofline": rf,
               "e2e": {"value": e2e_value, "unit": "matrices/s", "h2d_bytes_per_step": int(n * 9 * 8),
                       "d2h_bytes_per_step": int(n * (9 + 81 + 729) * 8),
                       "ms_per_step": e2e_ms, "api": "gmf_cuda_eval_host",
                       "timer": "host wall clock around the synchronous call"},
               "gpu_launches": args.steps * launches_per_call(args.kind, n),
               "clocks": clk.summary()}
    del dA, dF, dJ, dH
    torch.cuda.empty_cache()
    cpu_log = None
    if rank == 0 and not args.no_cpu:
        call = CpuCall("gmf_eval", kind, args.alpha, group_sample(X, args.cpu_sample), 2)
        out["cpu_baseline"] = cpu_log = cpu_baseline(call, args.cpu_budget,
                                                     f"gmf_eval {args.kind} order 2 on the C1 groups")
    want = set(args.sections.split(",")) if args.sections else None
    run = lambda name: rank == 0 and (want is None or name in want)
    if run("c1_kinds"):
        section(out, "c1_kinds", lambda: c1_kinds(lib, args, dev, pk, X))
    if run("smf_c0"):
        section(out, "smf_c0", lambda: smf_c0(lib, args, dev, pk))
    if run("mixed") and not args.no_mixed:
        section(out, "mixed", lambda: mixed_sweep(lib, args, dev, pk))
    if run("mixed_gmf") and not args.no_mixed:
        section(out, "mixed_gmf", lambda: mixed_gmf(lib, args, dev, pk, cpu_log))
    if run("adjoint") and not args.no_adjoint:
        section(out, "adjoint", lambda: adjoint_vs_materialised(lib, args, dev, pk))
    if run("tangent") and not args.no_adjoint:
        section(out, "tangent", lambda: tangent_vs_materialised(lib, args, dev, pk, X))
    if run("batched") and not args.no_batched:
        section(out, "batched", lambda: batched_c3(lib, args, dev, pk))
    if rank == 0:
        out["pipe_peaks_tflops"] = {"fp64": pk.fp64, "fp32": pk.fp32}
        print(json.dumps(out), flush=True)


# DRAM bytes per matrix of the ordered gmf_kernel<LOG, 2> launch from one ncu capture at n = 262144 on the same
# workload (132.8 MB read + 1915.7 MB written for 259 584 matrices; the algorithmic bytes are 6624 per matrix, the
# extra bytes are the partial sectors at the ends of the rows the ordered launch scatters)
NCU_DRAM_BYTES_PER_MATRIX = (132.77e6 + 1915.68e6) / 259584
NCU_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the ordered gmf_kernel<LOG,2> launch at "
                      "n=262144 (2048.4 MB), scaled by n (profiles/gmf_kernel_log_o2_c1.md)")


def launches_per_call(kind, n):
    """kernels one order-2 gmf_cuda_eval call launches: key, scan, scatter, the ordered launch and the tail launch
    (every kind with 2^15 <= n <= 2^31 - 1), else one plain launch"""
    return 5 if (1 << 15) <= n <= (1 << 31) - 1 else 1


# ------------------------------------------------------------------------------------------------ ncu count pass
def count_pass(args):
    """one launch per configuration at a small size, each preceded by a one-element torch kernel as a separator, for
    an ncu capture of the FP64 / FP32 instruction and DRAM counters; the configurations and their sizes go to
    stdout as JSON (tag, matrices), in launch order"""
    import torch

    import matfun_gb300
    from matfun_gb300 import workloads as w
    lib = matfun_gb300.load()
    dev = torch.device("cuda", 0)
    sep = torch.zeros(1, device=dev)
    manifest = []

    def one(tag, n, fn):
        torch.cuda.synchronize()
        sep.add_(1.0)
        r = fn()
        if r not in (0, None):
            raise RuntimeError(f"{tag}: returned {r}")
        torch.cuda.synchronize()
        manifest.append({"tag": tag, "n": n})

    ng = 1 << 16
    Xg = torch.from_numpy(w.c1_gmf_groups(ng, seed=1).reshape(ng, 9)).to(dev)
    out = [torch.empty((ng, k), dtype=torch.float64, device=dev) for k in (9, 81, 729)]
    for name in ("log", "exp", "sqrt"):
        one(f"gmf/{name}/2/f64", ng, lambda: lib.gmf_cuda_eval(KINDS[name], 0.0, ng, Xg.data_ptr(),
                                                               *[t.data_ptr() for t in out], None))
    X32 = Xg.float()
    o32 = [t.float() for t in out]
    for name, kind, alpha in (("log", 1, 0.0), ("exp", 0, 0.0), ("sqrt", 3, 0.0), ("pow0.3", 2, 0.3)):
        one(f"gmf/{name}/2/f32", ng, lambda: lib.gmf_cuda_eval_f32(kind, alpha, ng, X32.data_ptr(),
                                                                   *[t.data_ptr() for t in o32], None))
    F, G, K = (torch.empty((ng, k), dtype=torch.float64, device=dev) for k in (9, 9, 81))
    one("gmf/log/tangent/f64", ng, lambda: lib.gmf_cuda_tangent(1, 0.0, ng, Xg.data_ptr(), F.data_ptr(), G.data_ptr(),
                                                                K.data_ptr(), None))
    del out, o32, X32, F, G, K
    torch.cuda.empty_cache()
    n0 = args.smf_n
    V0 = torch.from_numpy(w.c0_smf_spd(n0)).to(dev)
    s0 = [torch.empty((n0, k), dtype=torch.float64, device=dev) for k in (6, 36, 216)]
    one("smf/log/2/f64/c0", n0, lambda: lib.smf_cuda_eval(1, 0.0, n0, V0.data_ptr(), *[t.data_ptr() for t in s0],
                                                          None))
    del V0, s0
    n2 = 1 << 18
    x32 = torch.from_numpy(w.c2_smf_spd(n2, seed=2)).to(dev)
    x64 = x32.double()
    rng = np.random.default_rng(2)
    for name, kind in (("exp", 0), ("log", 1), ("sqrt", 3), ("pow", 2)):
        alpha = float(rng.uniform(0.1, 0.9)) if kind == 2 else 0.0
        for order in (0, 1, 2):
            for dt, x, fn in (("f32", x32, lib.smf_cuda_eval_f32), ("f64", x64, lib.smf_cuda_eval)):
                o = [torch.empty((n2, 6 ** (k + 1)), dtype=x.dtype, device=dev) for k in range(order + 1)]
                p = [t.data_ptr() for t in o] + [None] * (2 - order)
                one(f"smf/{name}/{order}/{dt}", n2, lambda: fn(kind, alpha, n2, x.data_ptr(), *p, None))
                del o
    del x32, x64
    torch.cuda.empty_cache()
    na = 1 << 18
    for fam, kind, alpha, name in (("smf", 1, 0.0, "log"), ("gmf", 2, 0.3, "pow0.3")):
        Ah = w.c0_smf_spd(na, seed=4, as_voigt=False) if fam == "smf" else w.c1_gmf_groups(2 * na, seed=4)[:na]
        A = torch.from_numpy(np.ascontiguousarray(Ah)).to(dev)
        W, V = torch.randn_like(A), torch.randn_like(A)
        o = [torch.empty_like(A) for _ in range(3)]
        for dt in ("f64", "f32"):
            Ax, Wx, Vx = (A, W, V) if dt == "f64" else (A.float(), W.float(), V.float())
            ox = o if dt == "f64" else [t.float() for t in o]
            fn = {("smf", "f64"): lib.smf_cuda_adjoint, ("gmf", "f64"): lib.gmf_cuda_adjoint,
                  ("smf", "f32"): lib.smf_cuda_adjoint_f32, ("gmf", "f32"): lib.gmf_cuda_adjoint_f32}[(fam, dt)]
            one(f"{fam}/{name}/vjp/{dt}", na, lambda: fn(kind, alpha, na, Ax.data_ptr(), Wx.data_ptr(), None, None,
                                                        ox[0].data_ptr(), None, None, None))
            one(f"{fam}/{name}/hvp/{dt}", na, lambda: fn(kind, alpha, na, Ax.data_ptr(), Wx.data_ptr(), Vx.data_ptr(),
                                                        None, None, ox[1].data_ptr(), ox[2].data_ptr(), None))
        del A, W, V, o
        torch.cuda.empty_cache()
    print(json.dumps({"count_pass": manifest}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kind", default="log", choices=["exp", "log", "sqrt"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--cpu-sample", type=int, default=1 << 15)
    ap.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of CPU work for the headline baseline")
    ap.add_argument("--cpu-budget-section", type=float, default=2.0)
    ap.add_argument("--cpu-budget-row", type=float, default=0.5)
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
    ap.add_argument("--smf-n", type=int, default=1 << 16, help="matrices of the C0 section (smf log order 2)")
    ap.add_argument("--sections", default="",
                    help="comma-separated sections to run after the headline (default: all): c1_kinds, smf_c0, mixed, "
                         "mixed_gmf, adjoint, tangent, batched")
    ap.add_argument("--count-pass", action="store_true",
                    help="one small launch per configuration (for ncu counters), no timing")
    args = ap.parse_args()
    args.alpha = 0.0  # exp, log; sqrt is mapped to pow 0.5 inside the library
    if args.count_pass:
        count_pass(args)
        return
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

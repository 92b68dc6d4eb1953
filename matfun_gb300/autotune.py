"""Autotuner of the batched persistent launch: CTAs per SM (1..4), the request layout (as given / longest work
first) and the tile geometry of the symmetric family (64 or 128 matrices per tile of 128 threads; the general family's
tile is 128), chosen by timing matfun_cuda_batched_run on a request mix, and kept in a JSON cache keyed by the GPU
name and the mix.  `apply()` sets the cached choice (matfun_cuda_batched_tune, matfun_cuda_batched_tune_tiles);
`tune(reqs)` measures and stores it.  `tune_smf_f32(x)` / `apply_smf_f32()` do the same for the store path of the
FP32 symmetric kernels (per-entry stores or TMA boxes of two widths, matfun_cuda_smf_f32_tune).

The cache lives in $MATFUN_AUTOTUNE_CACHE or ~/.cache/matfun_gb300/autotune.json.
"""
import json
import os

import torch

from . import batched
from ._lib import load

DEFAULT = {"ctas_per_sm": 2, "longest_first": 1, "smf_tile": 128}


def _set(lib, choice):
    lib.matfun_cuda_batched_tune(int(choice["ctas_per_sm"]), int(choice["longest_first"]))
    lib.matfun_cuda_batched_tune_tiles(int(choice.get("smf_tile", 128)))


def cache_path():
    return os.environ.get("MATFUN_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "matfun_gb300",
                                                                   "autotune.json")


def _key(reqs):
    fams = sorted({(r.c.family, r.c.order, r.c.dtype) for r in reqs})
    return f"{torch.cuda.get_device_name()}|" + ",".join(f"{f}{o}{d}" for f, o, d in fams)


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def apply(reqs=None):
    """set the cached choice for this GPU (and mix, if given); the default without an entry"""
    c = _load()
    choice = c.get(_key(reqs), None) if reqs is not None else None
    if choice is None:
        name = torch.cuda.get_device_name()
        choice = next((v for k, v in c.items() if k.startswith(name + "|")), DEFAULT)
    _set(load(), choice)
    return choice


def tune(reqs, reps=3, candidates=None, save=True):
    """time every candidate on the mix, keep the fastest (and store it); returns (choice, timings in ms)"""
    lib = load()
    cands = candidates or [{"ctas_per_sm": c, "longest_first": lf, "smf_tile": t}
                           for c in (1, 2, 3, 4) for lf in (1, 0) for t in (128, 64)]
    times = {}
    for cand in cands:
        _set(lib, cand)
        plan = batched.Plan(reqs)  # the layout and the tiles are fixed when the table is built
        plan.run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.run()
        e1.record()
        e1.synchronize()
        times[json.dumps(cand, sort_keys=True)] = e0.elapsed_time(e1) / reps
        del plan
    best = json.loads(min(times, key=times.get))
    _set(lib, best)
    if save:
        c = _load()
        c[_key(reqs)] = best
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(c, f, indent=1, sort_keys=True)
    return best, times


# ---- store path of the FP32 symmetric kernels (Voigt layout, orders 1 and 2)
SMF_F32_PATHS = {0: "per-entry stores", 1: "TMA boxes of 32 rows x 128 B", 2: "TMA boxes of 32 rows x 64 B",
                 3: "TMA boxes of 32 rows x 64 B, 14 CTAs per SM at order 2"}


def tune_smf_f32(x, kind=1, alpha=0.0, reps=3, save=True):
    """time smf_cuda_eval_f32 on the FP32 Voigt matrices `x` (a CUDA tensor, n x 6) through every store path at
    orders 1 and 2, keep the fastest per order (matfun_cuda_smf_f32_tune) and store it under the GPU's name; returns
    (choice {order: path}, timings {order: {path: ms}})"""
    lib = load()
    n = x.shape[0]
    st = torch.cuda.current_stream().cuda_stream
    choice, times = {}, {}
    for order in (1, 2):
        out = [torch.empty((n, 6 ** (k + 1)), dtype=torch.float32, device=x.device) for k in range(order + 1)]
        ptr = [t.data_ptr() for t in out] + [None] * (2 - order)
        times[order] = {}
        for path in SMF_F32_PATHS:
            lib.matfun_cuda_smf_f32_tune(order, path)
            assert lib.smf_cuda_eval_f32(kind, alpha, n, x.data_ptr(), *ptr, st) == 0
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                lib.smf_cuda_eval_f32(kind, alpha, n, x.data_ptr(), *ptr, st)
            e1.record()
            e1.synchronize()
            times[order][path] = e0.elapsed_time(e1) / reps
        choice[order] = min(times[order], key=times[order].get)
        lib.matfun_cuda_smf_f32_tune(order, choice[order])
        del out
    if save:
        c = _load()
        c[f"{torch.cuda.get_device_name()}|smf_f32"] = {str(k): v for k, v in choice.items()}
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(c, f, indent=1, sort_keys=True)
    return choice, times


def apply_smf_f32():
    """set the cached store paths of the FP32 symmetric kernels for this GPU (the library's default without one)"""
    c = _load().get(f"{torch.cuda.get_device_name()}|smf_f32")
    if c:
        lib = load()
        for order, path in c.items():
            lib.matfun_cuda_smf_f32_tune(int(order), int(path))
    return c

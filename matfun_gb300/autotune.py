"""Autotuner of the batched persistent launch: CTAs per SM (1..4), the request layout (as given / longest work
first) and the tile geometry of the symmetric family (64 or 128 matrices per tile of 128 threads; the general family's
tile is 128), chosen by timing matfun_cuda_batched_run on a request mix, and kept in a JSON cache keyed by the GPU
name and the mix.  `apply()` sets the cached choice (matfun_cuda_batched_tune, matfun_cuda_batched_tune_tiles);
`tune(reqs)` measures and stores it.

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

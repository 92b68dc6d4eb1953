"""Batched evaluation of many requests in one persistent launch (matfun_cuda_batched of include/matfun_cuda.h).

    reqs = [batched.request("gmf", "log", A1, order=2), batched.request("smf", "sqrt", V2, order=1), ...]
    batched.run(reqs)                          # one launch; outputs in reqs[i].F / .J / .H
    plan = batched.Plan(reqs)                  # table uploaded once
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g): plan.run()       # capturable: cursor reset + launch only
    g.replay()
"""
import ctypes

import torch

from ._lib import KINDS, Request, load

FAMILIES = {"smf_voigt": 0, "smf": 1, "gmf": 2}


class BatchRequest:
    """one request with its device output tensors; family "smf_voigt" (Voigt vectors), "smf" (symmetric matrices)
    or "gmf"; FP32 input selects the mixed-precision path"""

    def __init__(self, family, kind, x, order=0, alpha=None):
        if family not in FAMILIES:
            raise ValueError(f"family must be one of {sorted(FAMILIES)}")
        if kind not in KINDS:
            raise ValueError(f"unknown function {kind!r}")
        if not x.is_cuda or x.dtype not in (torch.float32, torch.float64):
            raise TypeError("expected a float32 / float64 CUDA tensor")
        self.x = x.contiguous()
        nin = 6 if family == "smf_voigt" else 9
        if self.x.shape[-1] != nin and tuple(self.x.shape[-2:]) != (3, 3):
            raise ValueError("bad input shape")
        self.n = self.x.numel() // nin
        nf = nin
        dt = self.x.dtype
        self.F = torch.empty((self.n, nf), dtype=dt, device=x.device)
        self.J = torch.empty((self.n, nf * nf), dtype=dt, device=x.device) if order >= 1 else None
        self.H = torch.empty((self.n, nf ** 3), dtype=dt, device=x.device) if order >= 2 else None
        p = lambda t: None if t is None else t.data_ptr()
        self.c = Request(FAMILIES[family], KINDS[kind], order, 1 if dt == torch.float32 else 0, float(alpha or 0.0),
                         self.n, p(self.x), p(self.F), p(self.J), p(self.H))


def request(family, kind, x, order=0, alpha=None):
    return BatchRequest(family, kind, x, order, alpha)


def _array(reqs):
    arr = (Request * len(reqs))()
    for i, r in enumerate(reqs):
        arr[i] = r.c
    return arr


def run(reqs, stream=None):
    """all requests in one launch on the current (or given) torch stream"""
    s = torch.cuda.current_stream() if stream is None else stream
    r = load().matfun_cuda_batched(ctypes.cast(_array(reqs), ctypes.c_void_p), len(reqs), s.cuda_stream)
    if r != 0:
        raise RuntimeError(f"matfun_cuda_batched returned {r}")


class Plan:
    """the request table uploaded once; run() can be captured in a CUDA graph"""

    def __init__(self, reqs):
        self.reqs = list(reqs)  # keeps the tensors alive
        self.h = ctypes.c_void_p()
        r = load().matfun_cuda_batched_plan(ctypes.cast(_array(self.reqs), ctypes.c_void_p), len(self.reqs),
                                            ctypes.byref(self.h))
        if r != 0:
            raise RuntimeError(f"matfun_cuda_batched_plan returned {r}")

    def run(self, stream=None):
        s = torch.cuda.current_stream() if stream is None else stream
        r = load().matfun_cuda_batched_run(self.h, s.cuda_stream)
        if r != 0:
            raise RuntimeError(f"matfun_cuda_batched_run returned {r}")

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            load().matfun_cuda_batched_free(self.h)
            self.h = ctypes.c_void_p()

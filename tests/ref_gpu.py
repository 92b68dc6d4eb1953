"""ctypes driver of oracle/ref_gpu_timer.so: the reference's own CUDA kernels (compiled for sm_103a from its sources
into oracle/_ref/matfun_cuda_ref.cubin) launched on device buffers.  Test and benchmark infrastructure only."""
import ctypes
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "matfun_cuda_ref.cubin")
TIMER = os.path.join(ROOT, "oracle", "ref_gpu_timer.so")
_lib = None


def available():
    return os.path.exists(CUBIN) and os.path.exists(TIMER)


def load():
    """the launcher with the cubin loaded into the current (torch primary) context"""
    global _lib
    if _lib is None:
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        lib = ctypes.CDLL(TIMER)
        lib.refgpu_load.argtypes = [ctypes.c_char_p]
        for fn in (lib.refgpu_gmf, lib.refgpu_smf):
            fn.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int64] + [ctypes.c_void_p] * 5
            fn.restype = ctypes.c_int
        r = lib.refgpu_load(CUBIN.encode())
        if r != 0:
            raise RuntimeError(f"refgpu_load failed ({r})")
        _lib = lib
    return _lib

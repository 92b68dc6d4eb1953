"""calls of the C ABI on device buffers (torch for allocation and copies only)"""
import numpy as np


def gpu_call(fam, kind, alpha, X, order, nf, stream=None):
    """(return code, F, J, H) of smf_cuda_eval / smf_cuda_eval_matrix / gmf_cuda_eval on n inputs X (n, 6 or 9)"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    fn = {"smf_eval": lib.smf_cuda_eval, "smf_eval_matrix": lib.smf_cuda_eval_matrix, "gmf_eval": lib.gmf_cuda_eval}[fam]
    X = np.ascontiguousarray(X, dtype=np.float64)
    n = len(X)
    dX = torch.from_numpy(X).cuda()
    dF = torch.full((n, nf), -7.0, dtype=torch.float64, device="cuda")
    dJ = torch.full((n, nf * nf), -7.0, dtype=torch.float64, device="cuda") if order >= 1 else None
    dH = torch.full((n, nf ** 3), -7.0, dtype=torch.float64, device="cuda") if order >= 2 else None
    p = lambda t: None if t is None else t.data_ptr()
    st = torch.cuda.current_stream().cuda_stream if stream is None else stream
    r = fn(kind, float(alpha), n, p(dX), p(dF), p(dJ), p(dH), st)
    torch.cuda.synchronize()
    out = [None if t is None else t.cpu().numpy() for t in (dF, dJ, dH)]
    return (r, *out)

"""The XLA FFI custom-call handlers on the GPU: one call frame per custom call, as XLA issues it for matfun.jax
(x on XLA's stream, F / (F, J) / (F, J, H) results, attributes kind and alpha), for every family and order; the
results must be those of the C ABI entry points (the same kernels), also with batch dimensions of rank > 2."""
import ctypes as C

import numpy as np
import pytest

from tests import xla_ffi_frames as xf

pytestmark = pytest.mark.gpu

FAMS = {"voigt": ("smf_cuda_eval", (6,), 6), "matrix": ("smf_cuda_eval_matrix", (3, 3), 9),
        "general": ("gmf_cuda_eval", (3, 3), 9)}


def inputs(fam, batch, seed):
    import torch
    from matfun_gb300 import workloads as w
    n = int(np.prod(batch))
    if fam == "general":
        A = w.c1_gmf_groups(4 * ((n + 3) // 4), seed=seed)[:n]
    else:
        A = w.c0_smf_spd(n, seed=seed, as_voigt=(fam == "voigt"))
    return torch.from_numpy(np.ascontiguousarray(A)).cuda().reshape(*batch, *FAMS[fam][1])


@pytest.mark.parametrize("fam", list(FAMS))
@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("kind,alpha", [(1, 0.0), (2, 0.3), (0, 0.0)])
def test_handler_equals_c_abi(fam, order, kind, alpha):
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    raw = C.CDLL(matfun_gb300.library_path())
    entry, tail, nf = FAMS[fam]
    batch = (5, 7)
    x = inputs(fam, batch, seed=order + 3 * kind)
    n = int(np.prod(batch))
    shapes = [tail, tail * 2, tail * 3]
    outs = [torch.full((*batch, *shapes[k]), 5.0, dtype=torch.float64, device="cuda") for k in range(order + 1)]
    ref = [torch.full((n, nf ** (k + 1)), 7.0, dtype=torch.float64, device="cuda") for k in range(order + 1)]
    stream = torch.cuda.Stream()
    xla = xf.FakeXla(stream=stream.cuda_stream)
    cf, keep = xf.frame(xla, (xf.DT_F64, x.data_ptr(), tuple(x.shape)),
                        [(xf.DT_F64, o.data_ptr(), tuple(o.shape)) for o in outs], xf.std_attrs(kind, alpha))
    torch.cuda.synchronize()
    r = xf.handler(raw, xf.HANDLERS[fam][order])(C.addressof(cf))
    assert r is None, xla.errors
    stream.synchronize()
    p = [t.data_ptr() for t in ref] + [None] * (2 - order)
    assert getattr(lib, entry)(kind, alpha, n, x.data_ptr(), *p, None) == 0
    torch.cuda.synchronize()
    for o, rf in zip(outs, ref):
        a, b = o.reshape(n, -1).cpu().numpy(), rf.cpu().numpy()
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert np.array_equal(np.nan_to_num(a), np.nan_to_num(b))

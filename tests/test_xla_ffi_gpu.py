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


@pytest.mark.parametrize("fam,handler,entry", [("voigt", "SmfValueF32Cuda", "smf_cuda_eval_f32"),
                                               ("matrix", "SmfMatrixValueF32Cuda", "smf_cuda_eval_matrix_f32"),
                                               ("general", "GmfValueF32Cuda", "gmf_cuda_eval_f32")])
@pytest.mark.parametrize("order", [0, 2])
def test_f32_handlers_equal_c_abi(fam, handler, entry, order):
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    raw = C.CDLL(matfun_gb300.library_path())
    _, tail, nf = FAMS[fam]
    batch = (3, 11)
    x = inputs(fam, batch, seed=7).float()
    n = int(np.prod(batch))
    shapes = [tail, tail * 2, tail * 3]
    outs = [torch.full((*batch, *shapes[k]), 5.0, dtype=torch.float32, device="cuda") for k in range(order + 1)]
    ref = [torch.full((n, nf ** (k + 1)), 7.0, dtype=torch.float32, device="cuda") for k in range(order + 1)]
    xla = xf.FakeXla()
    cf, keep = xf.frame(xla, (xf.DT_F32, x.data_ptr(), tuple(x.shape)),
                        [(xf.DT_F32, o.data_ptr(), tuple(o.shape)) for o in outs], xf.std_attrs(1, 0.0))
    assert xf.handler(raw, handler)(C.addressof(cf)) is None, xla.errors
    p = [t.data_ptr() for t in ref] + [None] * (2 - order)
    assert getattr(lib, entry)(1, 0.0, n, x.data_ptr(), *p, None) == 0
    torch.cuda.synchronize()
    for o, rf in zip(outs, ref):
        assert torch.equal(torch.nan_to_num(o.reshape(n, -1)), torch.nan_to_num(rf))


@pytest.mark.parametrize("fam", ["smf", "gmf"])
@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("mask", [2, 1 | 2 | 4 | 8])
def test_adjoint_handlers_equal_c_abi(fam, dt, mask):
    """the adjoint handlers (outputs F, J^T W, J V, W.H.V selected by a bit mask) give the results of
    smf_cuda_adjoint / gmf_cuda_adjoint (and the FP32 forms) on the same buffers"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    raw = C.CDLL(matfun_gb300.library_path())
    tdt, xdt = (torch.float64, xf.DT_F64) if dt == "f64" else (torch.float32, xf.DT_F32)
    batch = (4, 9)
    A = inputs("general" if fam == "gmf" else "matrix", batch, seed=3).to(tdt)
    g = torch.Generator(device="cuda").manual_seed(4)
    W = torch.randn(A.shape, dtype=tdt, device="cuda", generator=g)
    V = torch.randn(A.shape, dtype=tdt, device="cuda", generator=g) if mask & 12 else torch.empty(0, dtype=tdt,
                                                                                                    device="cuda")
    n = int(np.prod(batch))
    sel = [b for b in range(4) if mask >> b & 1]
    outs = [torch.full_like(A, 5.0) for _ in sel]
    name = ("Smf" if fam == "smf" else "Gmf") + "Adjoint" + ("F32" if dt == "f32" else "") + "Cuda"
    xla = xf.FakeXla()
    cf, keep = xf.frame3(xla, [(xdt, t.data_ptr(), tuple(t.shape)) for t in (A, W, V)],
                         [(xdt, o.data_ptr(), tuple(o.shape)) for o in outs], xf.adjoint_attrs(2, 0.3, mask))
    assert xf.handler(raw, name)(C.addressof(cf)) is None, xla.errors
    ref = [torch.full_like(A, 7.0) if mask >> b & 1 else None for b in range(4)]
    fn = getattr(lib, f"{fam}_cuda_adjoint" + ("_f32" if dt == "f32" else ""))
    p = lambda t: None if t is None else t.data_ptr()
    assert fn(2, 0.3, n, A.data_ptr(), W.data_ptr(), p(V) if V.numel() else None, *map(p, ref), None) == 0
    torch.cuda.synchronize()
    for o, b in zip(outs, sel):
        assert torch.equal(torch.nan_to_num(o), torch.nan_to_num(ref[b]))


@pytest.mark.parametrize("mask", [4, 1 | 2 | 4])
def test_tangent_handler_equals_c_abi(mask):
    """GmfTangentCuda (F, G = J^T F, K = J^T J + F : H selected by a bit mask) gives the results of gmf_cuda_tangent"""
    import torch

    import matfun_gb300
    lib = matfun_gb300.load()
    raw = C.CDLL(matfun_gb300.library_path())
    batch = (4, 9)
    A = inputs("general", batch, seed=5)
    n = int(np.prod(batch))
    shapes = {0: A.shape, 1: A.shape, 2: (*batch, 3, 3, 3, 3)}
    sel = [b for b in range(3) if mask >> b & 1]
    outs = [torch.full(shapes[b], 5.0, dtype=torch.float64, device="cuda") for b in sel]
    xla = xf.FakeXla()
    cf, keep = xf.frame3(xla, [(xf.DT_F64, A.data_ptr(), tuple(A.shape))],
                         [(xf.DT_F64, o.data_ptr(), tuple(o.shape)) for o in outs], xf.adjoint_attrs(1, 0.0, mask))
    assert xf.handler(raw, "GmfTangentCuda")(C.addressof(cf)) is None, xla.errors
    ref = [torch.full(shapes[b], 7.0, dtype=torch.float64, device="cuda") if mask >> b & 1 else None for b in range(3)]
    p = lambda t: None if t is None else t.data_ptr()
    assert lib.gmf_cuda_tangent(1, 0.0, n, A.data_ptr(), *map(p, ref), None) == 0
    torch.cuda.synchronize()
    for o, b in zip(outs, sel):
        assert torch.equal(torch.nan_to_num(o), torch.nan_to_num(ref[b]))

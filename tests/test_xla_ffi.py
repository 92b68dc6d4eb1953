"""The XLA FFI custom-call handlers (SmfValueCuda ... GmfValueJacHessCuda) without a GPU: the metadata query, the
API version, and every malformed call frame the reference's binding rejects (cuda/src/matfun_cuda.cu:220-261, the
checks of its XLA FFI binding), called with frames built the way XLA builds them.  Only paths that end before a
launch run here; the launches are in test_xla_ffi_gpu.py.  The layout of the frame structures is pinned against the
XLA FFI header the reference vendors, where the reference tree is present (oracle/Makefile.ref, ffi-abi)."""
import ctypes as C
import os
import subprocess

import pytest

from tests import xla_ffi_frames as xf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import matfun_gb300
    if not os.path.exists(matfun_gb300.library_path()):
        from matfun_gb300 import build
        build.build_cuda()
    return C.CDLL(matfun_gb300.library_path())


def call(lib, name, cf):
    return xf.handler(lib, name)(C.addressof(cf))


def voigt_frame(xla, **kw):
    dims = kw.pop("dims", (4, 6))
    dtype = kw.pop("dtype", xf.DT_F64)
    nret = kw.pop("nret", 1)
    attrs = kw.pop("attrs", xf.std_attrs(1, 0.0))
    rets = kw.pop("rets", [(xf.DT_F64, 8, dims)] * nret)
    return xf.frame(xla, (dtype, 16, dims), rets, attrs, **kw)


def test_api_version_and_symbols(lib):
    lib.smf_xla_ffi_api_version.restype = C.c_int
    assert lib.smf_xla_ffi_api_version() == 1  # XLA FFI API 0.1, major * 1000 + minor
    for names in xf.HANDLERS.values():
        for nm in names:
            assert hasattr(lib, nm)


def test_metadata_query(lib):
    """a frame carrying the metadata extension asks for the API version and traits; nothing else is read"""
    for names in xf.HANDLERS.values():
        for nm in names:
            xla = xf.FakeXla()
            md = xf.Metadata(struct_size=C.sizeof(xf.Metadata))
            ext = xf.MetadataExt(xf.Ext(C.sizeof(xf.MetadataExt), xf.EXT_METADATA, None), C.pointer(md))
            cf = xf.CallFrame(struct_size=xf.CALL_FRAME_SIZE, api=C.pointer(xla.api), stage=0)
            cf.extension_start = C.cast(C.pointer(ext), C.POINTER(xf.Ext))
            assert call(lib, nm, cf) is None
            assert (md.api_version.major_version, md.api_version.minor_version, md.traits) == (0, 1, 0)
            assert xla.errors == []


def expect_invalid(lib, name, cf, keep, xla, text):
    r = call(lib, name, cf)
    assert r is not None and r == len(xla.errors), "handler must return the error it created"
    errc, msg = xla.errors[-1]
    assert errc == xf.ERR_INVALID_ARGUMENT and text in msg, msg


def test_malformed_frames_are_invalid_arguments(lib):
    X = xf.FakeXla
    cases = [
        ("struct size", dict(struct_size=xf.CALL_FRAME_SIZE + 8), "XLA_FFI_CallFrame size"),
        ("stage", dict(stage=0), "execution stage"),
        ("input dtype", dict(dtype=xf.DT_F32), "dtype"),
        ("argument type", dict(arg_types=[7]), "argument type"),
        ("Voigt shape", dict(dims=(4, 5)), "(..., 6)"),
        ("scalar input", dict(dims=()), "(..., 6)"),
        ("no results", dict(nret=0), "(F, J, H)"),
        ("four results", dict(nret=4), "(F, J, H)"),
        ("result dtype", dict(rets=[(xf.DT_F64, 8, (4, 6)), (xf.DT_F32, 8, (4, 36))]), "result"),
        ("kind type", dict(attrs={"kind": (xf.ATTR_SCALAR, xf.DT_F64, C.c_double(1.0)),
                                  "alpha": (xf.ATTR_SCALAR, xf.DT_F64, C.c_double(0.0))}), "kind"),
        ("alpha missing", dict(attrs={"kind": (xf.ATTR_SCALAR, xf.DT_S64, C.c_int64(1)),
                                      "beta": (xf.ATTR_SCALAR, xf.DT_F64, C.c_double(0.0))}), "alpha"),
        ("three attributes", dict(attrs={**xf.std_attrs(1, 0.0), "x": (xf.ATTR_SCALAR, xf.DT_S64, C.c_int64(0))}),
         "number of attributes"),
        ("invalid kind", dict(attrs=xf.std_attrs(7, 0.0)), "invalid kind"),
        ("huge kind", dict(attrs=xf.std_attrs(2 ** 40, 0.0)), "invalid kind"),
        ("pow without alpha", dict(attrs=xf.std_attrs(2, 0.0)), "invalid kind or alpha"),
        ("negative kind", dict(attrs=xf.std_attrs(-3, 0.5)), "invalid kind"),
    ]
    for label, kw, text in cases:
        xla = X()
        cf, keep = voigt_frame(xla, **kw)
        expect_invalid(lib, "SmfValueCuda", cf, keep, xla, text)
    # matrix families want (..., 3, 3)
    for nm in ("SmfMatrixValueCuda", "GmfValueJacHessCuda"):
        xla = X()
        cf, keep = xf.frame(xla, (xf.DT_F64, 16, (4, 9)), [(xf.DT_F64, 8, (4, 9))], xf.std_attrs(0, 0.0))
        expect_invalid(lib, nm, cf, keep, xla, "(..., 3, 3)")
    # two arguments
    xla = X()
    cf, keep = voigt_frame(xla)
    cf.args.size = 2
    expect_invalid(lib, "GmfValueCuda", cf, keep, xla, "number of arguments")


def test_empty_batch_succeeds_without_launch(lib):
    """an input with zero matrices is a valid call that launches nothing (smf_cuda_eval with n = 0)"""
    for fam, dims in (("voigt", (0, 6)), ("matrix", (0, 3, 3)), ("general", (2, 0, 3, 3))):
        for order, nm in enumerate(xf.HANDLERS[fam]):
            xla = xf.FakeXla()
            cf, keep = xf.frame(xla, (xf.DT_F64, 16, dims), [(xf.DT_F64, 8, dims)] * (order + 1),
                                xf.std_attrs(3, 0.0))
            assert call(lib, nm, cf) is None and xla.errors == []


def test_handler_reports_a_refused_launch_as_internal(lib):
    """an input beyond the reference's grid limit is a launch the library refuses: INTERNAL, no device work"""
    xla = xf.FakeXla()
    dims = (2 ** 31, 2 ** 6, 6)  # 2^37 Voigt vectors: beyond 32 * (2^31 - 1)
    cf, keep = xf.frame(xla, (xf.DT_F64, 16, dims), [(xf.DT_F64, 16, dims)], xf.std_attrs(1, 0.0))
    r = xf.handler(lib, "SmfValueCuda")(C.addressof(cf))
    assert r is not None and xla.errors[-1][0] == xf.ERR_INTERNAL


def test_frame_layout_pinned_to_the_vendored_xla_header():
    """compile-time comparison of matfun_gb300/csrc/xla_ffi_abi.h with the XLA FFI C API header that the reference
    vendors (sizes, field offsets, structure-size macros, enumerated values); needs the reference tree"""
    from matfun_gb300 import build
    ref = build.reference_root()
    if ref is None:
        pytest.skip("reference tree not present")
    r = subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), f"REF={ref}", "ffi-abi"],
                       cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr



def test_adjoint_frames_checked_before_launch(lib):
    """the additional adjoint handlers: shapes, directions, the output mask and the result count are checked before
    anything runs; an empty batch succeeds without a launch"""
    A = (xf.DT_F64, 16, (4, 3, 3))
    Z = (xf.DT_F64, 24, (0,))
    at = xf.adjoint_attrs
    cases = [
        ("no outputs", "SmfAdjointCuda", [A, A, Z], at(1, 0.0, 0), [], "outputs"),
        ("mask beyond 4 bits", "SmfAdjointCuda", [A, A, Z], at(1, 0.0, 16), [A], "outputs"),
        ("result count", "GmfAdjointCuda", [A, A, Z], at(1, 0.0, 2 | 4), [A], "one result per selected output"),
        ("W of another shape", "SmfAdjointCuda", [A, (xf.DT_F64, 24, (5, 3, 3)), Z], at(1, 0.0, 2), [A], "shape of A"),
        ("A not (..., 3, 3)", "GmfAdjointCuda", [(xf.DT_F64, 16, (4, 9)), A, Z], at(1, 0.0, 1), [A], "(..., 3, 3)"),
        ("J^T W without W", "SmfAdjointCuda", [A, Z, Z], at(1, 0.0, 2), [A], "invalid kind or alpha"),
        ("F64 buffers to an F32 handler", "GmfAdjointF32Cuda", [A, A, Z], at(1, 0.0, 1), [A], "dtype"),
        ("two arguments", "SmfAdjointCuda", [A, A], at(1, 0.0, 1), [A], "number of arguments"),
    ]
    for label, nm, args, attrs, rets, text in cases:
        xla = xf.FakeXla()
        cf, keep = xf.frame3(xla, args, rets, attrs)
        assert call(lib, nm, cf) is not None, label
        assert xla.errors[-1][0] == xf.ERR_INVALID_ARGUMENT and text in xla.errors[-1][1], (label, xla.errors[-1])
    E = (xf.DT_F64, 16, (0, 3, 3))
    for nm in ("SmfAdjointCuda", "GmfAdjointCuda"):
        xla = xf.FakeXla()
        cf, keep = xf.frame3(xla, [E, E, E], [E, E], at(1, 0.0, 1 | 8))
        assert call(lib, nm, cf) is None and xla.errors == []


def test_tangent_frames_checked_before_launch(lib):
    """GmfTangentCuda: the argument shape, the output mask (K required), the result count and shapes are checked
    before anything runs; an empty batch succeeds without a launch"""
    A = (xf.DT_F64, 16, (4, 3, 3))
    K = (xf.DT_F64, 16, (4, 3, 3, 3, 3))
    at = xf.adjoint_attrs
    cases = [
        ("no K", [A], at(1, 0.0, 1 | 2), [A, A], "outputs"),
        ("mask beyond 3 bits", [A], at(1, 0.0, 8 | 4), [K], "outputs"),
        ("result count", [A], at(1, 0.0, 1 | 4), [K], "one result per selected output"),
        ("K of A's shape", [A], at(1, 0.0, 4), [A], "K 9 times"),
        ("A not (..., 3, 3)", [(xf.DT_F64, 16, (4, 9))], at(1, 0.0, 4), [K], "(..., 3, 3)"),
        ("F32 buffer", [(xf.DT_F32, 16, (4, 3, 3))], at(1, 0.0, 4), [K], "dtype"),
        ("pow without alpha", [A], at(2, 0.0, 4), [K], "invalid kind or alpha"),
    ]
    for label, args, attrs, rets, text in cases:
        xla = xf.FakeXla()
        cf, keep = xf.frame3(xla, args, rets, attrs)
        assert call(lib, "GmfTangentCuda", cf) is not None, label
        assert xla.errors[-1][0] == xf.ERR_INVALID_ARGUMENT and text in xla.errors[-1][1], (label, xla.errors[-1])
    E = (xf.DT_F64, 16, (0, 3, 3))
    xla = xf.FakeXla()
    cf, keep = xf.frame3(xla, [E], [E, (xf.DT_F64, 16, (0, 9, 9))], at(1, 0.0, 1 | 4))
    assert call(lib, "GmfTangentCuda", cf) is None and xla.errors == []

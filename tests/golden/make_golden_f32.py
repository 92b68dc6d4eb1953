"""Golden cases of the FP32 (mixed-precision) entry points, derived from the reference's golden cases.

    python tests/golden/make_golden_f32.py          (needs oracle/liboracle.so: __graft_entry__.build())

Takes every case of tests/golden/cases_smf.npz and cases_gmf.npz (the reference's testdata/cases.txt and
cases_general.txt: smf in the Voigt layout, gmf in the matrix layout) whose input fits FP32 comfortably (every entry 0
or 1e-30 <= |x| <= 1e30; this drops the 1e+-100-scaled cases), rounds the input to FP32 and evaluates F, J, H of it
with the FP64 oracle (the CPU restatement of the reference algorithm) on those rounded values. Cases whose FP64
results leave FP32's range (|x| > 1e30 anywhere) are dropped too. Writes tests/golden/cases_smf_f32.npz and
cases_gmf_f32.npz: x (float32 inputs), F, J, H (float64 expected values of those inputs), kind, alpha and the per-case
tolerance on max|x - ref| / max|ref| of each of F, J, H, which is the error statement of the FP32 path for that kind
(tol below). The FP32 path's own rounding of its inputs is thereby excluded; what is tested is its arithmetic.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# max |x - ref| / max |ref| per case and output (F, J, H): 2e-6 for every family and kind, except large exponents
# (pow with alpha > 8, here 60.5), where the assembly of J and H from the FP32-rounded divided differences cancels
# (the Newton-form coefficients of x^60.5 grow like binomial(60.5, k)): smf 4e-6; gmf 2e-4 (J up to 1.6e-5, H up to
# 1.0e-4 on these cases, F 5e-8)


def tol(fam, kind, alpha):
    if kind == 2 and alpha > 8:
        return 4e-6 if fam == "smf" else 2e-4
    return 2e-6


def derive(fam, fn, src, dst, nf):
    sys.path.insert(0, ROOT)
    from tests import oracle_lib as ol
    g = np.load(os.path.join(HERE, src))
    x = g["x"]
    ax = np.abs(x)
    keep = np.all((ax == 0) | ((ax >= 1e-30) & (ax <= 1e30)), axis=1)
    x32 = np.where(keep[:, None], x, 0.0).astype(np.float32)
    out = {k: [] for k in ("kind", "alpha", "tol", "x", "F", "J", "H")}
    for i in np.where(keep)[0]:
        kind, alpha = int(g["kind"][i]), float(g["alpha"][i])
        r, F, J, H = ol.call(ol.oracle(), fn, kind, alpha, x32[i:i + 1].astype(np.float64), 2, nf)
        assert r == 0
        big = max(np.nanmax(np.abs(a), initial=0.0) for a in (F, J, H))
        if big > 1e30:
            continue
        for k, v in (("kind", kind), ("alpha", alpha), ("tol", tol(fam, kind, alpha)), ("x", x32[i]), ("F", F[0]),
                     ("J", J[0]), ("H", H[0])):
            out[k].append(v)
    np.savez_compressed(os.path.join(HERE, dst), kind=np.array(out["kind"], np.int32), alpha=np.array(out["alpha"]),
                        tol=np.array(out["tol"]), x=np.array(out["x"], np.float32),
                        **{k: np.array(out[k]) for k in "FJH"})
    print(f"{src}: {len(out['kind'])} of {len(x)} cases -> {dst}")


if __name__ == "__main__":
    derive("smf", "smf_eval", "cases_smf.npz", "cases_smf_f32.npz", 6)
    derive("gmf", "gmf_eval", "cases_gmf.npz", "cases_gmf_f32.npz", 9)

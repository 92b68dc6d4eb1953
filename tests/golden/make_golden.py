"""Converts the reference's cross-language golden cases into compact fixtures for the parity tests.

    python tests/golden/make_golden.py REFERENCE_ROOT     (the reference source tree)

Reads testdata/cases.txt (smf, Voigt layout: kind alpha tol v[6] F[6] J[36] H[216]) and testdata/cases_general.txt
(gmf, matrix layout: kind alpha tol A[9] F[9] J[81] H[729]) of the reference -- F, J, H computed by the reference's
FP64 C kernel, with a per-case tolerance on max|x - ref| / max|ref| for each of F, J, H -- and writes
tests/golden/cases_smf.npz and tests/golden/cases_gmf.npz (float64 arrays kind, alpha, tol, x, F, J, H).
The reference tree is only needed to regenerate the fixtures, never by the tests.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def convert(src, dst, nin, nf):
    rows = np.loadtxt(src, comments="#")
    nj, nh = nf * nf, nf * nf * nf
    assert rows.shape[1] == 3 + nin + nf + nj + nh, rows.shape
    o = 3
    parts = {}
    for name, w in (("x", nin), ("F", nf), ("J", nj), ("H", nh)):
        parts[name] = rows[:, o:o + w]
        o += w
    np.savez_compressed(dst, kind=rows[:, 0].astype(np.int32), alpha=rows[:, 1], tol=rows[:, 2], **parts)
    print(f"{src}: {len(rows)} cases -> {dst} ({os.path.getsize(dst) / 1e6:.2f} MB)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py REFERENCE_ROOT")
    ref = sys.argv[1]
    convert(os.path.join(ref, "testdata", "cases.txt"), os.path.join(HERE, "cases_smf.npz"), 6, 6)
    convert(os.path.join(ref, "testdata", "cases_general.txt"), os.path.join(HERE, "cases_gmf.npz"), 9, 9)

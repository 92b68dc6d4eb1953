"""comparison helpers shared by the tests"""
import re

import numpy as np


def maxrel(a, b):
    """max |a - b| / max |b| over entries, skipping positions where both are NaN (a NaN on one side only: inf),
    as the reference's CUDA test (cuda/tests/test_cuda_api.cu:15-23)"""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    both = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b)
    d[both] = 0.0
    d = np.where(np.isnan(d), np.inf, d)
    s = np.max(np.abs(np.where(np.isnan(b), 0.0, b)), initial=0.0)
    return float(np.max(d, initial=0.0) / max(s, 1e-300))


def maxrel_rows(a, b):
    """per-row version of maxrel for (n, k) arrays"""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b)
    d[both] = 0.0
    d = np.where(np.isnan(d), np.inf, d)
    s = np.max(np.abs(np.where(np.isnan(b), 0.0, b)), axis=1)
    return np.max(d, axis=1) / np.maximum(s, 1e-300)


FLT_MAX, FLT_MIN = 3.4028234663852886e38, 1.1754943508222875e-38


def maxrel_rows_fp32(got, ref):
    """per-matrix errors (max |x - ref| / max |ref| of each row) over the rows whose reference lies within FP32's
    normal range (FP32 storage cannot hold the others) and is not all NaN; NaN positions must agree row by row"""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    smax = np.max(np.abs(np.where(np.isnan(ref), 0.0, ref)), axis=1)
    keep = (smax <= FLT_MAX) & (smax >= FLT_MIN) & ~np.isnan(ref).all(axis=1)
    return maxrel_rows(got[keep], ref[keep])


def random_general(n, seed=99):
    """4 n general 3x3 matrices in four families: diagonalisable with spectra over e^+-3, complex pairs of modulus
    e^+-2 at random angles beside a real eigenvalue, Jordan blocks (double and triple eigenvalues of modulus e^+-2
    with unit-scale couplings) perturbed by 1e-14 .. 1e-2, each similarity-transformed by S = N(0, 1) + U(0.5, 4) I;
    and I + 0.5 N(0, 1)"""
    rng = np.random.default_rng(seed)

    def conj(M):
        S = rng.standard_normal((len(M), 3, 3)) + rng.uniform(0.5, 4, (len(M), 1, 1)) * np.eye(3)
        return S @ M @ np.linalg.inv(S)

    D = np.zeros((n, 3, 3))
    D[:, [0, 1, 2], [0, 1, 2]] = np.exp(rng.uniform(-3, 3, (n, 3)))
    r, t = np.exp(rng.uniform(-2, 2, n)), rng.uniform(-3.14, 3.14, n)
    M = np.zeros((n, 3, 3))
    M[:, 0, 0] = M[:, 1, 1] = r * np.cos(t)
    M[:, 0, 1], M[:, 1, 0] = -r * np.sin(t), r * np.sin(t)
    M[:, 2, 2] = np.exp(rng.uniform(-2, 2, n))
    J = np.zeros((n, 3, 3))
    J[:, [0, 1, 2], [0, 1, 2]] = np.exp(rng.uniform(-2, 2, n))[:, None]
    J[:, 0, 1], J[:, 1, 2] = rng.uniform(0, 2, n), rng.uniform(0, 2, n)
    J += 10 ** rng.uniform(-14, -2, (n, 1, 1)) * rng.standard_normal((n, 3, 3))
    return np.concatenate([conj(D), conj(M), conj(J), np.eye(3) + 0.5 * rng.standard_normal((n, 3, 3))])


def header_functions(path):
    """names of the functions an include/*.h declares"""
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*([A-Za-z_][A-Za-z_0-9]*)\s*\(", src, flags=re.M)


def voigt_to_matrix(v):
    """(n, 6) Voigt vectors -> (n, 3, 3) symmetric matrices"""
    A = np.empty(v.shape[:-1] + (3, 3))
    A[..., 0, 0], A[..., 1, 1], A[..., 2, 2] = v[..., 0], v[..., 1], v[..., 2]
    A[..., 0, 1] = A[..., 1, 0] = v[..., 3]
    A[..., 0, 2] = A[..., 2, 0] = v[..., 4]
    A[..., 1, 2] = A[..., 2, 1] = v[..., 5]
    return A


def near_degenerate_f32():
    """the near-degenerate set: FP32 matrices within 2^-30 .. 2^-70 of a multiple of I, c (I + 2^-e S) with S
    symmetric and of zero diagonal (the deviator exactly representable in FP32); row 29913 of C0 (n = 65536, seed 4),
    whose FP32 eigenvectors came out of smf_eigsys_ff 0.6 % from orthonormal on GB300 (F 3e-3 from the oracle); and
    row 31949 of C0 (n = 50000, seed 6), a triple eigenvalue rounded to FP32, whose pair's Jacobi block squared into
    FP32's subnormal range before that block was scaled (H 2e-2 from the oracle)"""
    from matfun_gb300 import workloads as w
    rng = np.random.default_rng(29913)
    parts = [w.c0_smf_spd(65536, seed=4, as_voigt=False)[29913:29914],
             w.c0_smf_spd(50000, seed=6, as_voigt=False)[31949:31950]]
    for e in (30, 39, 41, 52, 60, 70):
        c = np.exp(rng.uniform(-2, 2, 256))
        S = rng.standard_normal((256, 3, 3))
        S = S + S.transpose(0, 2, 1)
        S[:, [0, 1, 2], [0, 1, 2]] = 0.0
        parts.append(c[:, None, None] * (np.eye(3) + 2.0 ** -e * S))
    return np.concatenate(parts).astype(np.float32)


def build_host_math(src, out_dir, opt="-O2"):
    """compile tests/host_math/<src> (kernel headers built for the host) into a shared library in out_dir with g++;
    None where g++ or the CUDA headers are missing"""
    import os
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if cxx is None or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        return None
    out = os.path.join(str(out_dir), os.path.splitext(src)[0] + ".so")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "host_math", src)
    r = subprocess.run([cxx, "-std=c++17", opt, "-fPIC", "-shared", "-I" + inc, path, "-o", out],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return out

"""Seeded synthetic inputs of the benchmark configurations (shapes, sizes and value distributions of the reference's
stated workloads; no external data).

    c0_smf_spd(n, seed)      SPD matrices A = Q diag(lam) Q^T, Q Haar, ln lam ~ U(-1, 1); 10% with two equal and 2%
                             with three equal eigenvalues; Voigt vectors (n, 6)
    c1_gmf_groups(n, seed)   general matrices (n, 3, 3) in four equal groups: I + 0.3 N(0,1) (real spectra);
                             R(theta) diag(s) with theta ~ U(-3, 3) about a random axis, ln s ~ U(-0.5, 0.5) (complex
                             pairs); shear I + gamma e1 e2^T, gamma ~ U(-2, 2) (defective); the shears perturbed entrywise
                             by a relative 1e-10 N(0,1) (near-confluent)
"""
import numpy as np


def haar(rng, n):
    """n Haar-random orthogonal 3x3 matrices (QR of Gaussian matrices with the sign of diag(R) fixed)"""
    Z = rng.standard_normal((n, 3, 3))
    Q, R = np.linalg.qr(Z)
    d = np.sign(np.diagonal(R, axis1=1, axis2=2))
    d[d == 0] = 1.0
    return Q * d[:, None, :]


def voigt(A):
    return np.stack([A[..., 0, 0], A[..., 1, 1], A[..., 2, 2], A[..., 0, 1], A[..., 0, 2], A[..., 1, 2]], axis=-1)


def c0_smf_spd(n, seed=0, as_voigt=True):
    rng = np.random.default_rng(seed)
    Q = haar(rng, n)
    lam = np.exp(rng.uniform(-1.0, 1.0, (n, 3)))
    u = rng.uniform(size=n)
    dbl = u < 0.10
    tri = u >= 0.98
    lam[dbl, 1] = lam[dbl, 0]
    lam[tri, 1] = lam[tri, 0]
    lam[tri, 2] = lam[tri, 0]
    A = np.einsum("nij,nj,nkj->nik", Q, lam, Q)
    A = 0.5 * (A + A.transpose(0, 2, 1))
    return voigt(A) if as_voigt else A


def rotation(axis, theta):
    k = axis / np.linalg.norm(axis, axis=-1, keepdims=True)
    K = np.zeros(k.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2], K[..., 1, 2] = -k[..., 2], k[..., 1], -k[..., 0]
    K[..., 1, 0], K[..., 2, 0], K[..., 2, 1] = k[..., 2], -k[..., 1], k[..., 0]
    s, c = np.sin(theta)[..., None, None], np.cos(theta)[..., None, None]
    return np.eye(3) + s * K + (1.0 - c) * (K @ K)


def c1_gmf_groups(n, seed=1):
    rng = np.random.default_rng(seed)
    q = n // 4
    sizes = [q, q, q, n - 3 * q]
    g1 = np.eye(3) + 0.3 * rng.standard_normal((sizes[0], 3, 3))
    Rm = rotation(rng.standard_normal((sizes[1], 3)), rng.uniform(-3.0, 3.0, sizes[1]))
    g2 = Rm * np.exp(rng.uniform(-0.5, 0.5, (sizes[1], 1, 3)))
    g3 = np.tile(np.eye(3), (sizes[2], 1, 1))
    g3[:, 0, 1] = rng.uniform(-2.0, 2.0, sizes[2])
    src = g3[np.arange(sizes[3]) % sizes[2]]
    g4 = src * (1.0 + 1e-10 * rng.standard_normal((sizes[3], 3, 3)))
    return np.ascontiguousarray(np.concatenate([g1, g2, g3, g4]))


def c2_smf_spd(n, seed=2, as_voigt=True, dtype=np.float32):
    """SPD matrices with condition number log-uniform in [1, 1e6] and smallest eigenvalue gap log-uniform in
    [1e-12, 1] (relative), Haar eigenvectors, overall scale e^U(-1, 1); stored as `dtype`"""
    rng = np.random.default_rng(seed)
    Q = haar(rng, n)
    kappa = 10.0 ** rng.uniform(0.0, 6.0, n)
    gap = 10.0 ** rng.uniform(-12.0, 0.0, n)
    lo, hi = 1.0 / kappa, np.ones(n)
    near_lo = rng.uniform(size=n) < 0.5
    mid = np.where(near_lo, lo * (1.0 + gap), hi * (1.0 - gap))
    mid = np.clip(mid, lo, hi)
    lam = np.stack([lo, mid, hi], axis=1) * np.exp(rng.uniform(-1.0, 1.0, (n, 1)))
    A = np.einsum("nij,nj,nkj->nik", Q, lam, Q)
    A = 0.5 * (A + A.transpose(0, 2, 1))
    out = voigt(A) if as_voigt else A
    return np.ascontiguousarray(out.astype(dtype))

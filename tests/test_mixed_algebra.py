"""The linear algebra behind the mixed solver's p/v pass (CPU only).

Between FP64 hand-overs the pass forms v' = M p' (M = D^-1 A, the Jacobi-
scaled operator on the scaled Krylov vectors) without loading p, s at the
stencil points, from the two products already stored, t = M s and v = M p:

    p' = s - omega t + beta (p - omega v)
    M p' = w - omega M w,   w = t + beta v.

This pins the identity on a singular 7-point-like operator with the PPE's
structure (A 1 = 0, symmetric, negative semi-definite), in FP64 and in FP32
with the rounding the kernel sees.
"""
import numpy as np
import scipy.sparse as sp


def ppe_like(nx=12, ny=10, nz=8, seed=0):
    """Periodic in x and y, Neumann in z, positive couplings c_ij with
    A_ii = -sum_j c_ij: the structure of the PPE rows (PDE.F90:69-121)."""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    idx = np.arange(n).reshape(nz, ny, nx)
    rows, cols, vals = [], [], []
    for axis, periodic in ((2, True), (1, True), (0, False)):
        nb = np.roll(idx, -1, axis=axis)
        a, b = idx, nb
        if not periodic:
            a = np.take(idx, range(nz - 1), axis=0)
            b = np.take(idx, range(1, nz), axis=0)
        a, b = a.ravel(), b.ravel()
        c = rng.uniform(0.5, 2.0, a.size) * (4.0 if axis == 0 else 1.0)
        rows += [a, b]
        cols += [b, a]
        vals += [c, c]
    r, cl, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    off = sp.csr_matrix((v, (r, cl)), shape=(n, n))
    A = off - sp.diags(np.asarray(off.sum(axis=1)).ravel())
    return A


def test_operator_has_the_ppe_structure():
    A = ppe_like()
    assert abs(A @ np.ones(A.shape[0])).max() < 1e-12
    assert abs(A - A.T).max() < 1e-15


def test_recurrence_identity_in_fp64():
    A = ppe_like()
    dinv = 1.0 / A.diagonal()
    M = lambda x: dinv * (A @ x)  # noqa: E731
    rng = np.random.default_rng(1)
    n = A.shape[0]
    s, p = rng.standard_normal(n), rng.standard_normal(n)
    t, v = M(s), M(p)
    for beta, om in ((0.7, 1.3), (-0.2, 0.05), (3.0, -0.9)):
        p_new = s - om * t + beta * (p - om * v)
        w = t + beta * v
        direct, rec = M(p_new), w - om * M(w)
        assert np.linalg.norm(direct - rec) <= 1e-13 * np.linalg.norm(direct)


def test_recurrence_error_in_fp32_is_rounding_sized():
    """In FP32, with t and v rounded as stored, the recurrence and the
    direct product differ by FP32 rounding amplified by |M| (tens of ulp
    relative), not by anything structural."""
    A = ppe_like()
    dinv = (1.0 / A.diagonal()).astype(np.float32)
    A32 = A.astype(np.float32)
    M = lambda x: dinv * (A32 @ x)  # noqa: E731
    rng = np.random.default_rng(2)
    n = A.shape[0]
    s, p = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    t, v = M(s), M(p)
    beta, om = np.float32(0.8), np.float32(0.6)
    p_new = (s - om * t) + beta * (p - om * v)
    w = t + beta * v
    direct, rec = M(p_new), w - om * M(w)
    rel = np.linalg.norm((direct - rec).astype(np.float64)) / np.linalg.norm(direct.astype(np.float64))
    assert rel < 64 * np.finfo(np.float32).eps, rel
